"""Continuous-batching structure-function service on one GPU.

Requests (an image stack already in device memory, its lags and mode) arrive
at arbitrary times.  The server admits them in arrival order as soon as a
stream slot and enough device memory are free (first fit: a request that does
not fit yet does not block smaller ones behind it), launches each admitted
request on its own CUDA stream so that the work of all in-flight requests
overlaps on the device, and keeps every result resident on the device until
it is fetched.  Latency is measured from arrival to the completion of the
request's last kernel (a CUDA event).

The scheduling logic (`DdmServer`) talks to an executor with four methods
(`estimate_bytes`, `launch`, `done`, `finish`); `GpuExecutor` is the GB300 one,
and tests drive the same server with a fake executor on the CPU.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any, Deque, Dict, List, Optional

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

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


class GpuExecutor:
    """Runs requests on the GB300 through the C ABI, one stream per in-flight request."""

    def __init__(self, gpu_id: int = 0, precision: str = "ff", n_streams: int = 6):
        from ._fftopt import next_fast_len
        from . import _ddm_b200

        self._nfl = next_fast_len
        self._mod = _ddm_b200
        self.device = torch.device("cuda", int(gpu_id))
        self.precision = precision
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]
        self.free_streams = list(range(n_streams))
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

    def _plan(self, req: Request):
        T, H, W = tuple(req.frames.shape)
        nx, ny = self._nfl(W, "b200"), self._nfl(H, "b200")
        nt = self._nfl(2 * T, "b200") if req.mode == "fft" else 0
        frames, code = self._mod.frames_to_device(req.frames, self.device)
        plan = self._mod.DdmPlan(req.mode, T, H, W, code, req.lags, nx, ny, nt, req.window is not None,
                                 self.precision, self.device)
        return plan, frames

    def estimate_bytes(self, req: Request) -> int:
        import ctypes
        from . import _lib

        T, H, W = tuple(req.frames.shape)
        nx, ny = self._nfl(W, "b200"), self._nfl(H, "b200")
        nt = self._nfl(2 * T, "b200") if req.mode == "fft" else 0
        size = ctypes.c_size_t(0)
        _lib.check(_lib.load().fddm_b200_workspace_size(_lib.MODE[req.mode], _lib.PREC[self.precision], T, H, W,
                                                         len(req.lags), nx, ny, nt, int(req.window is not None),
                                                         ctypes.byref(size)))
        return int(size.value) + (len(req.lags) + 2) * ny * (nx // 2 + 1) * 8

    def has_slot(self) -> bool:
        return bool(self.free_streams)

    def launch(self, req: Request):
        k = self.free_streams.pop()
        stream = self.streams[k]
        with torch.cuda.stream(stream):
            plan, frames = self._plan(req)
            out = torch.empty(plan.out_shape, dtype=torch.float64, device=self.device)
            plan.run(frames, req.window, out, stream)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
        return {"k": k, "plan": plan, "out": out, "event": ev, "frames": frames}

    def done(self, handle) -> bool:
        return handle["event"].query()

    def finish(self, handle):
        """Release the stream slot and workspace; returns (result tensor, completion host time)."""
        self.free_streams.append(handle["k"])
        t = self.t0_host + self.t0_event.elapsed_time(handle["event"]) / 1000.0
        handle["plan"].workspace = None
        return handle["out"], t


class DdmServer:
    """Admission by device memory, continuous batching over stream slots, resident results."""

    def __init__(self, executor, memory_budget: int):
        self.ex = executor
        self.budget = int(memory_budget)
        self.in_use = 0
        self.queue: Deque[Request] = deque()
        self.inflight: List[tuple] = []
        self.finished: Dict[int, Request] = {}
        self.peak_inflight = 0

    def submit(self, req: Request) -> None:
        req.nbytes = self.ex.estimate_bytes(req)
        if req.nbytes > self.budget:
            raise RuntimeError("Not enough memory")  # could never be admitted
        self.queue.append(req)

    def step(self, now: float) -> List[Request]:
        """Retire finished work, then admit what fits; returns the requests completed in this step."""
        done = []
        still = []
        for req, h in self.inflight:
            if self.ex.done(h):
                req.result, req.completed = self.ex.finish(h)
                self.in_use -= req.nbytes
                self.finished[req.rid] = req
                done.append(req)
            else:
                still.append((req, h))
        self.inflight = still
        admitted = []
        for req in list(self.queue):
            if not self.ex.has_slot():
                break
            if self.in_use + req.nbytes <= self.budget:
                self.queue.remove(req)
                req.admitted = now
                self.in_use += req.nbytes
                self.inflight.append((req, self.ex.launch(req)))
                admitted.append(req)
        self.peak_inflight = max(self.peak_inflight, len(self.inflight))
        return done

    @property
    def idle(self) -> bool:
        return not self.queue and not self.inflight

    def fetch(self, rid: int):
        """The resident result of a finished request (and forget it)."""
        return self.finished.pop(rid).result


def replay(server: DdmServer, requests: List[Request], clock, poll_s: float = 2e-4) -> List[Request]:
    """Feed `requests` (sorted by `arrival`, seconds from start) to the server in real time."""
    t0 = clock()
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    out = []
    while pending or not server.idle:
        now = clock() - t0
        while pending and pending[0].arrival <= now:
            r = pending.popleft()
            r.arrival += t0
            server.submit(r)
        out.extend(server.step(clock()))
        if pending and server.idle:
            time.sleep(max(0.0, min(poll_s, pending[0].arrival - (clock() - t0))))
        else:
            time.sleep(poll_s)
    return out


def latency_summary(reqs: List[Request]) -> dict:
    lat = np.array([r.latency for r in reqs])
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "max_ms": float(lat.max() * 1e3), "n": int(len(lat))}
