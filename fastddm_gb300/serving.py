"""Continuous-batching structure-function service on one GPU.

Requests (an image stack already in device memory, its lags and mode) arrive
at arbitrary times.  Each step of the server retires finished work, then
admits queued requests in arrival order while a stream slot, the memory
budget, the workspace pool and the device's live free memory allow:

* a request that does not fit yet does not block later, smaller ones (first
  fit), until it has waited ``max_wait_s``: from then on nothing queued behind
  it is admitted ahead of it, so memory and slots drain towards it (aging: a
  large request cannot be passed indefinitely);
* the small requests admitted in one step run together as one batch (one
  persistent launch of the many-job temporal kernel, ``fastddm_gb300.batch``),
  the large ones each on a stream of their own; all of them overlap on the
  device;
* every workspace is carved from one preallocated device pool (no allocation
  on the device while requests are in flight, apart from the result buffers),
  and a result stays resident on the device until it is fetched.

A result is the same alone and in the mix: batches give the single-stack
result bit for bit.  Latency is measured from arrival to the completion of the
request's last kernel (a CUDA event).

The scheduling logic (`DdmServer`) talks to an executor with the methods
``estimate_bytes``, ``free_slots``, ``reserve``, ``release``, ``launch``,
``done`` and ``finish``; `GpuExecutor` is the GB300 one, and tests drive the
same server with a fake executor on the CPU.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass
from typing import Any, Deque, Dict, List, Optional, Tuple

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


@dataclass
class Request:
    """One structure-function job."""

    rid: int
    frames: Any                  # device tensor (T, H, W) or a host array
    lags: np.ndarray
    mode: str = "fft"
    window: Any = None
    arrival: float = 0.0         # host time (s)
    # filled by the server
    nbytes: int = 0
    admitted: float = float("nan")
    completed: float = float("nan")
    result: Any = None
    reservation: Any = None

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


class OffsetPool:
    """First-fit suballocator of byte ranges in one buffer (256-byte aligned)."""

    ALIGN = 256

    def __init__(self, nbytes: int):
        self.size = int(nbytes)
        self.free: List[Tuple[int, int]] = [(0, self.size)]  # (offset, length), sorted, coalesced

    def alloc(self, nbytes: int) -> Optional[int]:
        n = max(self.ALIGN, (int(nbytes) + self.ALIGN - 1) // self.ALIGN * self.ALIGN)
        for i, (off, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    del self.free[i]
                else:
                    self.free[i] = (off + n, ln - n)
                return off
        return None

    def release(self, off: int, nbytes: int) -> None:
        n = max(self.ALIGN, (int(nbytes) + self.ALIGN - 1) // self.ALIGN * self.ALIGN)
        self.free.append((off, n))
        self.free.sort()
        merged: List[Tuple[int, int]] = []
        for o, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((o, ln))
        self.free = merged

    @property
    def available(self) -> int:
        return sum(ln for _, ln in self.free)


class GpuExecutor:
    """Runs requests on the GB300 through the C ABI.

    Large requests run one per stream slot, small ones together as a batch in
    one slot.  Workspaces come from one device pool allocated up front
    (``pool_bytes``, default 60 % of the free memory); a request is admitted
    only if its workspace fits in the pool and its result buffer in the
    device's live free memory (``cudaMemGetInfo``, 90 % of it, the reference's
    margin).
    """

    BATCH_EXTRA = 1 << 20  # the many-job kernel's arguments and items, per request (bound)

    def __init__(self, gpu_id: int = 0, precision: str = "ff", n_streams: int = 6,
                 pool_bytes: Optional[int] = None):
        from ._fftopt import next_fast_len
        from . import _ddm_b200

        self._nfl = next_fast_len
        self._mod = _ddm_b200
        self.device = torch.device("cuda", int(gpu_id))
        self.precision = precision
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]
        self.free_streams = list(range(n_streams))
        if pool_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            pool_bytes = int(0.6 * free)
        self.pool_buffer = torch.empty(int(pool_bytes), dtype=torch.uint8, device=self.device)
        self.pool = OffsetPool(int(pool_bytes))
        self.pending_out = 0  # result bytes of reserved, not yet launched requests
        self.t0_host = None
        self.t0_event = None

    def clock_start(self) -> float:
        """Pair a host timestamp with a device event so completion events map to host time."""
        torch.cuda.synchronize(self.device)
        self.t0_event = torch.cuda.Event(enable_timing=True)
        self.t0_event.record(torch.cuda.current_stream(self.device))
        torch.cuda.synchronize(self.device)
        self.t0_host = time.perf_counter()
        return self.t0_host

    def _sizes(self, req: Request):
        T, H, W = tuple(req.frames.shape)
        nx, ny = self._nfl(W, "b200"), self._nfl(H, "b200")
        nt = self._nfl(2 * T, "b200") if req.mode == "fft" else 0
        return T, H, W, nx, ny, nt

    def _work_bytes(self, req: Request) -> int:
        import ctypes
        from . import _lib

        T, H, W, nx, ny, nt = self._sizes(req)
        size = ctypes.c_size_t(0)
        _lib.check(_lib.load().fddm_b200_workspace_size(_lib.MODE[req.mode], _lib.PREC[self.precision], T, H, W,
                                                         len(req.lags), nx, ny, nt, int(req.window is not None),
                                                         ctypes.byref(size)))
        return int(size.value)

    def _out_bytes(self, req: Request) -> int:
        T, H, W, nx, ny, nt = self._sizes(req)
        return (len(req.lags) + 2) * ny * (nx // 2 + 1) * 8

    def estimate_bytes(self, req: Request) -> int:
        return self._work_bytes(req) + self._out_bytes(req)

    def free_slots(self) -> int:
        return len(self.free_streams)

    def reserve(self, req: Request) -> bool:
        """Carve the request's workspace from the pool if it and its result buffer fit now.

        Free memory is read live (``cudaMemGetInfo`` plus what PyTorch's caching
        allocator holds unused), less the result buffers of requests reserved
        but not launched yet.
        """
        free, _ = torch.cuda.mem_get_info(self.device)
        free += torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        out = self._out_bytes(req)
        if self.pending_out + out > 0.9 * free:
            return False
        n = self._work_bytes(req) + self.BATCH_EXTRA
        off = self.pool.alloc(n)
        if off is None:
            return False
        req.reservation = (off, n)
        self.pending_out += out
        return True

    def release(self, req: Request) -> None:
        if req.reservation is not None:
            self.pool.release(*req.reservation)
            req.reservation = None

    def _launch_one(self, req: Request, stream, ws):
        T, H, W, nx, ny, nt = self._sizes(req)
        frames, code = self._mod.frames_to_device(req.frames, self.device)
        window = self._mod._window_to_device(req.window, self.device)
        plan = self._mod.DdmPlan(req.mode, T, H, W, code, req.lags, nx, ny, nt, window is not None,
                                 self.precision, self.device, workspace=ws)
        out = torch.empty(plan.out_shape, dtype=torch.float64, device=self.device)
        plan.run(frames, window, out, stream)
        return (plan, frames, window), out

    def launch(self, reqs: List[Request]):
        """One request, or several as one batch, on one stream slot.

        A batch needs one contiguous workspace: the requests' pooled ranges are
        swapped for one range of their total size.  If the pool has no such
        range the requests run one after another on the slot's stream, each in
        its own range.
        """
        k = self.free_streams.pop()
        stream = self.streams[k]
        self.pending_out = max(0, self.pending_out - sum(self._out_bytes(r) for r in reqs))
        span = None
        keep = []
        with torch.cuda.stream(stream):
            if len(reqs) > 1:
                need = sum(r.reservation[1] for r in reqs)
                off = self.pool.alloc(need)
                if off is not None:
                    from .batch import BatchPlan, make_job

                    for r in reqs:
                        self.release(r)
                    span = (off, need)
                    jobs = [make_job(r.frames, r.lags, mode=r.mode, window=r.window, device=self.device)
                            for r in reqs]
                    plan = BatchPlan(jobs, self.precision, self.device, workspace=self.pool_buffer[off:off + need])
                    plan.run(stream)
                    keep.append((plan, jobs))
                    outs = [j.out for j in jobs]
            if span is None:
                outs = []
                for r in reqs:
                    off, n = r.reservation
                    objs, out = self._launch_one(r, stream, self.pool_buffer[off:off + n])
                    keep.append(objs)
                    outs.append(out)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
        return {"k": k, "keep": keep, "span": span, "outs": outs, "event": ev, "reqs": reqs}

    def done(self, handle) -> bool:
        return handle["event"].query()

    def finish(self, handle) -> List[Tuple[Any, float]]:
        """Release the slot and the pooled workspaces; (result tensor, completion host time) per request."""
        self.free_streams.append(handle["k"])
        t = self.t0_host + self.t0_event.elapsed_time(handle["event"]) / 1000.0
        if handle["span"] is not None:
            self.pool.release(*handle["span"])
        for r in handle["reqs"]:
            self.release(r)
        handle["keep"] = None
        return [(o, t) for o in handle["outs"]]


class DdmServer:
    """Admission by memory, continuous batching over stream slots, aging, resident results."""

    def __init__(self, executor, memory_budget: int, max_wait_s: float = 0.25, small_bytes: Optional[int] = None,
                 max_batch: int = 8):
        self.ex = executor
        self.budget = int(memory_budget)
        self.max_wait_s = float(max_wait_s)
        # requests up to this size are launched together as batches (default: 1/64 of the budget)
        self.small_bytes = int(small_bytes) if small_bytes is not None else self.budget // 64
        self.max_batch = int(max_batch)
        self.in_use = 0
        self.queue: Deque[Request] = deque()
        self.inflight: List[tuple] = []
        self.finished: Dict[int, Request] = {}
        self.peak_inflight = 0
        self.batches = 0

    def submit(self, req: Request) -> None:
        req.nbytes = self.ex.estimate_bytes(req)
        if req.nbytes > self.budget:
            raise RuntimeError("Not enough memory")  # could never be admitted
        self.queue.append(req)

    def step(self, now: float) -> List[Request]:
        """Retire finished work, then admit what fits; returns the requests completed in this step."""
        done = []
        still = []
        for reqs, h in self.inflight:
            if self.ex.done(h):
                for req, (res, t) in zip(reqs, self.ex.finish(h)):
                    req.result, req.completed = res, t
                    self.in_use -= req.nbytes
                    self.finished[req.rid] = req
                    done.append(req)
            else:
                still.append((reqs, h))
        self.inflight = still

        # admission in arrival order; an aged request stops everything behind it
        admitted: List[Request] = []
        for req in list(self.queue):
            small = req.nbytes <= self.small_bytes
            slots_needed = sum(1 for r in admitted if r.nbytes > self.small_bytes) + (
                (sum(1 for r in admitted if r.nbytes <= self.small_bytes) + int(small) + self.max_batch - 1)
                // self.max_batch)
            if not small:
                slots_needed += 1
            if (slots_needed <= self._free_slots() and self.in_use + req.nbytes <= self.budget
                    and self.ex.reserve(req)):
                self.queue.remove(req)
                req.admitted = now
                self.in_use += req.nbytes
                admitted.append(req)
            elif now - req.arrival > self.max_wait_s:
                break
        # launch: large requests alone, small ones in batches of up to max_batch
        small = [r for r in admitted if r.nbytes <= self.small_bytes]
        for r in admitted:
            if r.nbytes > self.small_bytes:
                self.inflight.append(([r], self.ex.launch([r])))
        for i in range(0, len(small), self.max_batch):
            group = small[i:i + self.max_batch]
            if len(group) > 1:
                self.batches += 1
            self.inflight.append((group, self.ex.launch(group)))
        self.peak_inflight = max(self.peak_inflight, sum(len(r) for r, _ in self.inflight))
        return done

    def _free_slots(self) -> int:
        return self.ex.free_slots()

    @property
    def idle(self) -> bool:
        return not self.queue and not self.inflight

    def fetch(self, rid: int):
        """The resident result of a finished request (and forget it)."""
        return self.finished.pop(rid).result


def replay(server: DdmServer, requests: List[Request], clock, poll_s: float = 2e-4,
           deliver=None) -> List[Request]:
    """Feed `requests` (sorted by `arrival`, seconds from start) to the server in real time.

    `deliver(request)`, if given, is called for each completed request (a
    client taking its result, e.g. with ``server.fetch``); otherwise results
    stay resident on the device.
    """
    t0 = clock()
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    out = []
    while pending or not server.idle:
        now = clock() - t0
        while pending and pending[0].arrival <= now:
            r = pending.popleft()
            r.arrival += t0
            server.submit(r)
        finished = server.step(clock())
        if deliver is not None:
            for r in finished:
                deliver(r)
        out.extend(finished)
        if pending and server.idle:
            time.sleep(max(0.0, min(poll_s, pending[0].arrival - (clock() - t0))))
        else:
            time.sleep(poll_s)
    return out


def latency_summary(reqs: List[Request]) -> dict:
    lat = np.array([r.latency for r in reqs])
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "max_ms": float(lat.max() * 1e3), "n": int(len(lat))}
