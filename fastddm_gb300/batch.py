"""Many image stacks of uneven size and length in one call.

``ddm_batch`` validates every stack like ``ddm()`` (lags sorted and
deduplicated, lag 0 dropped with a warning, window shape checked) and runs all
of them as one prepared batch (``fddm_b200_batch_create`` / ``_launch``): one
workspace, spatial stages scheduled longest-first over library-owned streams,
and the temporal stages of all stacks in one persistent launch of the
many-job kernel per kernel variant and CTA size.  Each result equals the one
``ddm()`` gives for that stack alone.
"""

from __future__ import annotations

import ctypes
import warnings
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._config import DTYPE
from ._ddm_b200 import _TORCH_CODE, _window_to_device, frames_to_device
from ._fftopt import next_fast_len
from .imagestructurefunction import ImageStructureFunction

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def prepare_lags(lags, length: int) -> np.ndarray:
    """The lag handling of ``ddm()``: sorted, unique, validated, lag 0 dropped with a warning."""
    lags = np.array(sorted(set(lags)))
    if np.min(lags) < 0:
        raise RuntimeError("Negative lags are not possible.")
    if np.max(lags) > length - 1:
        raise RuntimeError(f"Lags larger than len(img_seq) - 1 = {length - 1} are not possible.")
    if lags[0] == 0:
        warnings.warn("Found 0 in lags. Removed for compatibility with other functions.")
        lags = lags[1:]
    return lags


@dataclass
class BatchJob:
    """One stack of a batch: device frames (any contiguous buffer) plus its parameters and output."""

    frames: "torch.Tensor"
    dtype_code: int
    shape: tuple  # (T, H, W) of the frames
    lags: np.ndarray
    mode: str
    nx: int
    ny: int
    nt: int
    window: Optional["torch.Tensor"] = None
    out: Optional["torch.Tensor"] = None
    _lags_c: np.ndarray = field(default=None, repr=False)


class BatchPlan:
    """Workspace, job table and prepared library plan for a fixed list of jobs; can be run repeatedly.

    Creating the plan queues every job's tables into the workspace and sets
    up the temporal stages (``fddm_b200_batch_create``); :meth:`run` enqueues
    the batch's kernels only (``fddm_b200_batch_launch``).  With
    ``graph=True`` the first run also captures that launch into a CUDA graph
    and every later run replays the graph.  `workspace` is an optional
    caller-owned device buffer of at least ``fddm_b200_batch_workspace_size``
    bytes.
    """

    def __init__(self, jobs: List[BatchJob], precision: str = "ff", device=None, graph: bool = False,
                 workspace: Optional["torch.Tensor"] = None):
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError("the b200 batch needs a CUDA device (GB300)")
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.precision = precision
        self.jobs = jobs
        self._plan = None
        self._use_graph = graph
        self._graph = None
        self._table = (_lib.Job * max(1, len(jobs)))()
        for i, j in enumerate(jobs):
            T, H, W = j.shape
            if j.out is None:
                j.out = torch.empty((len(j.lags) + 2, j.ny, j.nx // 2 + 1), dtype=torch.float64, device=self.device)
            j._lags_c = np.ascontiguousarray(j.lags, dtype=np.uint32)
            e = self._table[i]
            e.mode = _lib.MODE[j.mode]
            e.d_img_seq = j.frames.data_ptr()
            e.dtype = j.dtype_code
            e.length, e.height, e.width = T, H, W
            e.lags = j._lags_c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
            e.nlags = len(j._lags_c)
            e.nx, e.ny, e.nt = j.nx, j.ny, j.nt
            e.d_window = j.window.data_ptr() if j.window is not None else None
            e.d_out = j.out.data_ptr()
        lib = _lib.load()
        size = ctypes.c_size_t(0)
        with torch.cuda.device(self.device):
            _lib.check(lib.fddm_b200_batch_workspace_size(self._table, len(jobs), _lib.PREC[precision], ctypes.byref(size)))
            self.workspace_bytes = int(size.value)
            if workspace is not None:  # caller-owned (e.g. a slice of a preallocated pool)
                if workspace.numel() * workspace.element_size() < self.workspace_bytes:
                    raise ValueError(f"workspace too small: {self.workspace_bytes} bytes needed")
                self.workspace = workspace
            else:
                free, _ = torch.cuda.mem_get_info(self.device)
                cached = torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
                if self.workspace_bytes > 0.9 * (free + cached):
                    raise RuntimeError("Not enough memory")
                self.workspace = torch.empty(max(1, self.workspace_bytes), dtype=torch.uint8, device=self.device)
            handle = ctypes.c_void_p()
            self._stream = torch.cuda.current_stream(self.device)
            _lib.check(lib.fddm_b200_batch_create(self._table, len(jobs), _lib.PREC[precision],
                                                  self.workspace.data_ptr(), self.workspace_bytes,
                                                  self._stream.cuda_stream, ctypes.byref(handle)))
            self._plan = handle

    def _launch(self, stream) -> None:
        _lib.check(_lib.load().fddm_b200_batch_launch(self._plan, stream.cuda_stream))

    def run(self, stream=None) -> List["torch.Tensor"]:
        """Enqueue the whole batch on `stream` (default: current); returns the output tensors."""
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            if stream != self._stream:
                stream.wait_stream(self._stream)  # the tables queued at creation
            if not self._use_graph:
                self._launch(stream)
            else:
                if self._graph is None:
                    self._launch(stream)  # first run outside capture: kernel attributes and caches settle
                    g = torch.cuda.CUDAGraph()
                    side = torch.cuda.Stream(self.device)
                    side.wait_stream(stream)
                    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
                        self._launch(side)
                    stream.wait_stream(side)
                    self._graph = g
                with torch.cuda.stream(stream):
                    self._graph.replay()
        return [j.out for j in self.jobs]

    def __del__(self):
        if getattr(self, "_plan", None) is not None:
            try:
                _lib.load().fddm_b200_batch_destroy(self._plan)
            except Exception:  # interpreter shutdown: the library may already be unloaded
                pass
            self._plan = None


def make_job(img_seq, lags, *, mode: str = "fft", window=None, device=None) -> BatchJob:
    """Validate one stack as ``ddm()`` does and describe it as a batch job (frames copied to the device)."""
    if mode not in ("fft", "diff"):
        raise RuntimeError(f"Unknown mode '{mode}' selected. Only possible options are ['diff', 'fft'].")
    T, H, W = img_seq.shape
    lags = prepare_lags(lags, T)
    frames, code = frames_to_device(img_seq, device)
    wdev = _window_to_device(window, device)
    if wdev is not None and tuple(wdev.shape) != (H, W):
        raise RuntimeError(f"Window with shape {tuple(wdev.shape)} incompatible with image shape {(H, W)}.")
    nx, ny = next_fast_len(W, "b200"), next_fast_len(H, "b200")
    nt = next_fast_len(2 * T, "b200") if mode == "fft" else 0
    return BatchJob(frames, code, (T, H, W), lags, mode, nx, ny, nt, wdev)


def ddm_batch(stacks: Sequence, lags, *, mode: str = "fft", windows: Optional[Sequence] = None,
              precision: str = "ff", gpu_id: int = 0) -> List[ImageStructureFunction]:
    """Image structure functions of many stacks; `lags` is one iterable for all or one per stack."""
    device = torch.device("cuda", int(gpu_id))
    per_stack_lags = len(stacks) > 0 and len(lags) == len(stacks) and all(np.ndim(l) == 1 for l in lags)
    jobs = []
    for i, s in enumerate(stacks):
        lg = lags[i] if per_stack_lags else lags
        w = windows[i] if windows is not None else None
        jobs.append(make_job(s, lg, mode=mode, window=w, device=device))
    plan = BatchPlan(jobs, precision, device)
    outs = plan.run()
    torch.cuda.current_stream(device).synchronize()
    res = []
    for j, o in zip(jobs, outs):
        kx = 2 * np.pi * np.fft.fftfreq(j.nx)[: j.nx // 2 + 1]
        ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(j.ny))
        res.append(ImageStructureFunction(o.cpu().numpy(), kx.astype(DTYPE), ky.astype(DTYPE), j.nx, j.ny,
                                          j.lags.astype(DTYPE), _device_data=o))
    return res
