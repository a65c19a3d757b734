"""Scheduling logic of the serving loop, driven by a fake executor on the CPU."""

import numpy as np
import pytest

from fastddm_gb300.serving import DdmServer, Request, latency_summary


class FakeExecutor:
    """Each request needs `bytes` of memory and runs for `duration` fake seconds; a batch of requests
    runs for the longest of their durations on one slot."""

    def __init__(self, slots):
        self.slots = slots
        self.now = 0.0
        self.running = {}
        self.log = []

    def estimate_bytes(self, req):
        return req.frames["bytes"]

    def free_slots(self):
        return self.slots - len(self.running)

    def reserve(self, req):
        return True

    def release(self, req):
        pass

    def launch(self, reqs):
        h = object()
        self.running[h] = (reqs, self.now + max(r.frames["duration"] for r in reqs))
        self.log.append(("launch", [r.rid for r in reqs], self.now))
        return h

    def done(self, h):
        return self.running[h][1] <= self.now

    def finish(self, h):
        reqs, t = self.running.pop(h)
        return [(f"result-{r.rid}", t) for r in reqs]


def _req(rid, nbytes, duration, arrival):
    return Request(rid, {"bytes": nbytes, "duration": duration}, np.arange(1, 3), arrival=arrival)


def _drive(server, ex, reqs, dt=0.01, t_end=100.0):
    pending = sorted(reqs, key=lambda r: r.arrival)
    done = []
    while ex.now < t_end and (pending or not server.idle):
        while pending and pending[0].arrival <= ex.now:
            server.submit(pending.pop(0))
        done += server.step(ex.now)
        for _, (req, t) in list(ex.running.items()):
            assert server.in_use <= server.budget
        ex.now += dt
    return done


def test_all_requests_complete_within_memory_and_slots():
    ex = FakeExecutor(slots=3)
    server = DdmServer(ex, memory_budget=100, small_bytes=0)
    reqs = [_req(i, 30 + (i % 3) * 10, 0.05 + 0.01 * (i % 5), arrival=0.02 * i) for i in range(40)]
    done = _drive(server, ex, reqs)
    assert sorted(r.rid for r in done) == list(range(40))
    assert server.peak_inflight <= 3  # one request per slot when none counts as small
    assert all(r.completed >= r.arrival for r in done)
    assert server.fetch(5) == "result-5"


def test_requests_overlap_when_memory_allows():
    ex = FakeExecutor(slots=4)
    server = DdmServer(ex, memory_budget=100, small_bytes=0)
    reqs = [_req(i, 20, 1.0, arrival=0.0) for i in range(4)]
    done = _drive(server, ex, reqs)
    # all four were admitted together (continuous batching), so they finish together
    assert server.peak_inflight == 4
    assert max(r.completed for r in done) < 1.1


def test_first_fit_lets_small_requests_pass_a_waiting_large_one():
    ex = FakeExecutor(slots=4)
    server = DdmServer(ex, memory_budget=100, max_wait_s=10.0)
    reqs = [_req(0, 60, 1.0, 0.0), _req(1, 60, 1.0, 0.01), _req(2, 10, 0.1, 0.02)]
    done = {r.rid: r for r in _drive(server, ex, reqs)}
    # request 1 does not fit next to 0; request 2 does and finishes long before 0
    assert done[2].completed < done[0].completed < done[1].completed
    assert done[1].admitted >= done[0].completed - 1e-9


def test_aging_admits_a_large_request_despite_a_stream_of_small_ones():
    """Small requests keep arriving and would always fit beside each other; once the large request has
    waited max_wait_s nothing behind it is admitted ahead of it, so it runs within a bounded time."""
    ex = FakeExecutor(slots=4)
    server = DdmServer(ex, memory_budget=100, max_wait_s=0.5, small_bytes=0)
    reqs = [_req(0, 30, 1.0, 0.0), _req(1, 80, 0.5, 0.01)]
    reqs += [_req(2 + i, 30, 1.0, 0.02 + 0.1 * i) for i in range(60)]
    done = {r.rid: r for r in _drive(server, ex, reqs, t_end=200.0)}
    assert len(done) == 62
    assert done[1].admitted - done[1].arrival < 0.5 + 1.1  # its wait, then at most one run of the blockers
    without = DdmServer(FakeExecutor(slots=4), memory_budget=100, max_wait_s=1e9, small_bytes=0)
    ex2 = without.ex
    reqs2 = [_req(0, 30, 1.0, 0.0), _req(1, 80, 0.5, 0.01)] + [_req(2 + i, 30, 1.0, 0.02 + 0.1 * i)
                                                             for i in range(60)]
    done2 = {r.rid: r for r in _drive(without, ex2, reqs2, t_end=200.0)}
    assert done2[1].admitted > done[1].admitted + 2.0  # first fit alone starves it for much longer


def test_small_requests_admitted_together_share_one_slot():
    ex = FakeExecutor(slots=2)
    server = DdmServer(ex, memory_budget=100, small_bytes=10, max_batch=3)
    reqs = [_req(i, 5, 1.0, 0.0) for i in range(5)] + [_req(5, 40, 1.0, 0.0)]
    done = _drive(server, ex, reqs)
    assert len(done) == 6
    launches = [rids for kind, rids, t in ex.log if t == 0.0]
    # in arrival order the five small requests fill the two slots as batches of three and two;
    # the large one (a slot of its own) starts when a slot frees
    assert sorted(map(len, launches)) == [2, 3]
    assert server.batches == 2
    done = {r.rid: r for r in done}
    assert done[5].admitted >= 1.0 - 1e-9


def test_offset_pool_first_fit_and_coalescing():
    from fastddm_gb300.serving import OffsetPool

    pool = OffsetPool(4096)
    a = pool.alloc(1000)
    b = pool.alloc(1000)
    c = pool.alloc(1000)
    assert (a, b, c) == (0, 1024, 2048)
    assert pool.alloc(2000) is None
    pool.release(b, 1000)
    assert pool.alloc(1024) == 1024  # the hole is reused
    pool.release(a, 1000)
    pool.release(1024, 1024)
    pool.release(c, 1000)
    assert pool.free == [(0, 4096)] and pool.available == 4096


def test_request_larger_than_the_budget_is_refused():
    ex = FakeExecutor(slots=2)
    server = DdmServer(ex, memory_budget=100)
    with pytest.raises(RuntimeError, match="Not enough memory"):
        server.submit(_req(0, 101, 0.1, 0.0))


def test_latency_summary():
    rs = [Request(i, None, np.arange(1, 2), arrival=0.0) for i in range(100)]
    for i, r in enumerate(rs):
        r.completed = (i + 1) / 1000.0
    s = latency_summary(rs)
    assert abs(s["p50_ms"] - 50.5) < 1e-6 and s["n"] == 100
