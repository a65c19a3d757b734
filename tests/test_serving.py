"""Scheduling logic of the serving loop, driven by a fake executor on the CPU."""

import numpy as np
import pytest

from fastddm_gb300.serving import DdmServer, Request, latency_summary


class FakeExecutor:
    """Each request needs `bytes` of memory and runs for `duration` fake seconds."""

    def __init__(self, slots):
        self.slots = slots
        self.now = 0.0
        self.running = {}
        self.log = []

    def estimate_bytes(self, req):
        return req.frames["bytes"]

    def has_slot(self):
        return len(self.running) < self.slots

    def launch(self, req):
        h = object()
        self.running[h] = (req, self.now + req.frames["duration"])
        self.log.append(("launch", req.rid, self.now))
        return h

    def done(self, h):
        return self.running[h][1] <= self.now

    def finish(self, h):
        req, t = self.running.pop(h)
        return f"result-{req.rid}", t


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
    server = DdmServer(ex, memory_budget=100)
    reqs = [_req(i, 30 + (i % 3) * 10, 0.05 + 0.01 * (i % 5), arrival=0.02 * i) for i in range(40)]
    done = _drive(server, ex, reqs)
    assert sorted(r.rid for r in done) == list(range(40))
    assert server.peak_inflight <= 3
    assert all(r.completed >= r.arrival for r in done)
    assert server.fetch(5) == "result-5"


def test_requests_overlap_when_memory_allows():
    ex = FakeExecutor(slots=4)
    server = DdmServer(ex, memory_budget=100)
    reqs = [_req(i, 20, 1.0, arrival=0.0) for i in range(4)]
    done = _drive(server, ex, reqs)
    # all four were admitted together (continuous batching), so they finish together
    assert server.peak_inflight == 4
    assert max(r.completed for r in done) < 1.1


def test_first_fit_lets_small_requests_pass_a_waiting_large_one():
    ex = FakeExecutor(slots=4)
    server = DdmServer(ex, memory_budget=100)
    reqs = [_req(0, 60, 1.0, 0.0), _req(1, 60, 1.0, 0.01), _req(2, 10, 0.1, 0.02)]
    done = {r.rid: r for r in _drive(server, ex, reqs)}
    # request 1 does not fit next to 0; request 2 does and finishes long before 0
    assert done[2].completed < done[0].completed < done[1].completed
    assert done[1].admitted >= done[0].completed - 1e-9


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
