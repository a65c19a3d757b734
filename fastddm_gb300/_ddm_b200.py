"""The ``b200`` backend: image structure function on a GB300 through the C ABI.

These are the functions the reference's backend registry calls
(``src/python/_ddm.py:51-74``, dispatch at ``:175-188``), with the argument
lists of the ``cpp``/``cuda`` backends:

* ``ddm_fft_b200(img_seq, lags, nx, ny, nt, window, **kwargs)``
  (reference: ``src/python/_ddm_cpp.py:72`` ``ddm_fft_cpp``,
  ``src/python/_ddm_cuda.py:64`` ``ddm_fft_gpu``)
* ``ddm_diff_b200(img_seq, lags, nx, ny, window, **kwargs)``
  (reference: ``src/python/_ddm_cpp.py:21`` ``ddm_diff_cpp``,
  ``src/python/_ddm_cuda.py:16`` ``ddm_diff_gpu``)

Both return a new float64 array of shape ``(len(lags) + 2, ny, nx // 2 + 1)``:
the structure function for each lag, then the power spectrum, then the
variance, y-fftshifted.  Keyword arguments: ``gpu_id`` (device index, as the
``cuda`` backend), ``precision`` (``'ff'`` float-float, default; ``'f64'``;
``'f32'``).  PyTorch provides device memory and the stream; all arithmetic runs
in the library's sm_103a kernels, with no CPU fallback.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib

try:  # torch is plumbing only: device buffers and the CUDA stream
    import torch
except ImportError:  # pragma: no cover - the package needs torch for device memory
    torch = None


_TORCH_CODE = {}
if torch is not None:
    _TORCH_CODE = {
        torch.uint8: 0,
        torch.int16: 1,
        torch.int32: 3,
        torch.float32: 7,
        torch.float64: 8,
    }
    if hasattr(torch, "uint16"):
        _TORCH_CODE[torch.uint16] = 2
    if hasattr(torch, "uint32"):
        _TORCH_CODE[torch.uint32] = 4


def _require_torch():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("core='b200' needs a CUDA device (GB300) and PyTorch for device memory")


def _device(gpu_id) -> "torch.device":
    return torch.device("cuda", int(gpu_id))


def frames_to_device(img_seq, device) -> tuple["torch.Tensor", int]:
    """Copy (or adopt) an image sequence as a contiguous device tensor; returns (tensor, dtype code).

    64-bit integer inputs are converted to float64 first, like the reference's
    cast to its Scalar type (``src/cpp/ddm.cc:288-297``).
    """
    if torch is not None and isinstance(img_seq, torch.Tensor):
        t = img_seq
        if t.dtype in (torch.int64,) or (hasattr(torch, "uint64") and t.dtype == torch.uint64):
            t = t.to(torch.float64)
        if t.dtype not in _TORCH_CODE:
            raise TypeError(f"unsupported image dtype {t.dtype}")
        t = t.to(device).contiguous()
        return t, _TORCH_CODE[t.dtype]
    arr, code = host_frames(img_seq)
    raw = torch.from_numpy(arr.reshape(-1).view(np.uint8))
    dev = torch.empty(raw.numel(), dtype=torch.uint8, device=device)
    dev.copy_(raw)
    return dev, code


def host_frames(img_seq):
    """Host image sequence as a C-contiguous array (or CPU tensor) the library can read; returns (array, code)."""
    if torch is not None and isinstance(img_seq, torch.Tensor):
        t = img_seq
        if t.dtype == torch.int64 or (hasattr(torch, "uint64") and t.dtype == torch.uint64):
            t = t.to(torch.float64)
        if t.dtype not in _TORCH_CODE:
            raise TypeError(f"unsupported image dtype {t.dtype}")
        return t.contiguous(), _TORCH_CODE[t.dtype]
    arr = np.asarray(img_seq)
    if arr.ndim != 3:
        raise ValueError("img_seq must have shape (t, y, x)")
    if arr.dtype.name in ("int64", "uint64"):
        arr = arr.astype(np.float64)
    code = _lib.DTYPE_CODE.get(arr.dtype.name)
    if code is None or code in (5, 6):
        raise TypeError(f"unsupported image dtype {arr.dtype}")
    return np.ascontiguousarray(arr), code


def _host_ptr(a) -> int:
    return a.data_ptr() if (torch is not None and isinstance(a, torch.Tensor)) else a.ctypes.data


def _host_nbytes(a) -> int:
    return a.numel() * a.element_size() if (torch is not None and isinstance(a, torch.Tensor)) else a.nbytes


@dataclass
class DdmPlan:
    """Sizes, workspace and lags of one structure-function computation.

    A plan may be run many times on frames of the same shape and dtype; it owns
    its device workspace.
    """

    mode: str
    length: int
    height: int
    width: int
    dtype_code: int
    lags: np.ndarray
    nx: int
    ny: int
    nt: int
    has_window: bool
    precision: str = "ff"
    device: Optional["torch.device"] = None
    # a caller-owned device buffer to use as the workspace (e.g. a slice of a
    # preallocated pool); None: the plan allocates its own
    workspace: Optional["torch.Tensor"] = None

    def __post_init__(self):
        _require_torch()
        if self.mode not in _lib.MODE:
            raise RuntimeError(f"Unknown mode '{self.mode}'")
        if self.precision not in _lib.PREC:
            raise ValueError(f"precision must be one of {sorted(_lib.PREC)}")
        if self.device is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        lib = _lib.load()
        self._lags_c = np.ascontiguousarray(self.lags, dtype=np.uint32)
        size = ctypes.c_size_t(0)
        with torch.cuda.device(self.device):
            _lib.check(
                lib.fddm_b200_workspace_size(
                    _lib.MODE[self.mode], _lib.PREC[self.precision], self.length, self.height, self.width,
                    len(self._lags_c), self.nx, self.ny, self.nt, int(self.has_window), ctypes.byref(size),
                )
            )
            self.workspace_bytes = int(size.value)
            if self.workspace is not None:
                if self.workspace.numel() * self.workspace.element_size() < self.workspace_bytes:
                    raise ValueError(f"workspace too small: {self.workspace_bytes} bytes needed")
                return
            out_bytes = (len(self._lags_c) + 2) * self.ny * (self.nx // 2 + 1) * 8
            free, _ = torch.cuda.mem_get_info(self.device)
            cached = torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
            # the reference admits a job only within 90% of free device memory (memchk_gpu.cu:611-614)
            if self.workspace_bytes + out_bytes > 0.9 * (free + cached):
                raise RuntimeError("Not enough memory")
            self.workspace = torch.empty(max(self.workspace_bytes, 1), dtype=torch.uint8, device=self.device)

    @property
    def out_shape(self) -> tuple[int, int, int]:
        return (len(self._lags_c) + 2, self.ny, self.nx // 2 + 1)

    def run(self, frames: "torch.Tensor", window: Optional["torch.Tensor"], out: "torch.Tensor",
            stream: Optional["torch.cuda.Stream"] = None) -> "torch.Tensor":
        """Enqueue the computation on `stream` (default: the current stream); returns `out`."""
        lib = _lib.load()
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        if out.dtype != torch.float64 or tuple(out.shape) != self.out_shape or not out.is_contiguous():
            raise ValueError(f"out must be a contiguous float64 tensor of shape {self.out_shape}")
        lags_p = self._lags_c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        wptr = window.data_ptr() if window is not None else None
        with torch.cuda.device(self.device):
            if self.mode == "fft":
                code = lib.fddm_b200_ddm_fft(
                    frames.data_ptr(), self.dtype_code, self.length, self.height, self.width,
                    lags_p, len(self._lags_c), self.nx, self.ny, self.nt, wptr, out.data_ptr(),
                    self.workspace.data_ptr(), self.workspace_bytes, _lib.PREC[self.precision], stream.cuda_stream,
                )
            else:
                code = lib.fddm_b200_ddm_diff(
                    frames.data_ptr(), self.dtype_code, self.length, self.height, self.width,
                    lags_p, len(self._lags_c), self.nx, self.ny, wptr, out.data_ptr(),
                    self.workspace.data_ptr(), self.workspace_bytes, _lib.PREC[self.precision], stream.cuda_stream,
                )
        _lib.check(code)
        return out

    def run_from_host(self, host, frames_dev: "torch.Tensor", window: Optional["torch.Tensor"], out: "torch.Tensor",
                      host_out: Optional["torch.Tensor"] = None,
                      stream: Optional["torch.cuda.Stream"] = None) -> "torch.Tensor":
        """Enqueue the computation reading the frames from host memory (upload overlapped with compute).

        `host` must stay alive until the stream has finished; `host_out`, if
        given, receives the result (page-locked memory makes the copy async).
        `frames_dev` may be None for page-locked frames the row pass reads in
        place; the library refuses that (FDDM_ERR_INVALID, nothing queued) when
        they cannot be read in place.
        """
        lib = _lib.load()
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        if out.dtype != torch.float64 or tuple(out.shape) != self.out_shape or not out.is_contiguous():
            raise ValueError(f"out must be a contiguous float64 tensor of shape {self.out_shape}")
        lags_p = self._lags_c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        wptr = window.data_ptr() if window is not None else None
        hout = host_out.data_ptr() if host_out is not None else None
        with torch.cuda.device(self.device):
            code = lib.fddm_b200_ddm_from_host(
                _lib.MODE[self.mode], _host_ptr(host), self.dtype_code, self.length, self.height, self.width,
                lags_p, len(self._lags_c), self.nx, self.ny, self.nt,
                frames_dev.data_ptr() if frames_dev is not None else None, wptr, out.data_ptr(),
                hout, self.workspace.data_ptr(), self.workspace_bytes, _lib.PREC[self.precision], stream.cuda_stream,
            )
        _lib.check(code)
        return out


def _window_to_device(window, device) -> Optional["torch.Tensor"]:
    if window is None:
        return None
    if torch is not None and isinstance(window, torch.Tensor):
        if window.numel() == 0:
            return None
        return window.to(device=device, dtype=torch.float64).contiguous()
    w = np.asarray(window)
    if w.size == 0:
        return None
    return torch.from_numpy(np.ascontiguousarray(w, dtype=np.float64)).to(device)


def ddm_device(img_seq, lags: Sequence[int], nx: int, ny: int, nt: int, window=None, *, mode: str = "fft",
               precision: str = "ff", gpu_id: int = 0, host_out: bool = False):
    """Run the structure function; returns the device result tensor (and the host copy if `host_out`).

    Device-resident input (a CUDA tensor) is used in place.  Page-locked host
    input (a pinned CPU tensor whose rows are multiples of 16 bytes) is read in
    place by the row pass, without a device copy of the stack; other host
    input (numpy arrays, pageable tensors) is uploaded in chunks overlapped
    with the spatial FFTs.
    """
    _require_torch()
    device = _device(gpu_id)
    shape = tuple(img_seq.shape)
    if len(shape) != 3:
        raise ValueError("img_seq must have shape (t, y, x)")
    wdev = _window_to_device(window, device)
    if wdev is not None and tuple(wdev.shape) != shape[1:]:
        raise RuntimeError(f"Window with shape {tuple(wdev.shape)} incompatible with image shape {shape[1:]}.")
    on_device = torch is not None and isinstance(img_seq, torch.Tensor) and img_seq.is_cuda
    if on_device:
        frames, code = frames_to_device(img_seq, device)
    else:
        host, code = host_frames(img_seq)
    plan = DdmPlan(mode, shape[0], shape[1], shape[2], code, np.asarray(lags), int(nx), int(ny),
                   int(nt) if mode == "fft" else 0, wdev is not None, precision, device)
    out = torch.empty(plan.out_shape, dtype=torch.float64, device=device)
    hout = torch.empty(plan.out_shape, dtype=torch.float64, pin_memory=True) if host_out else None
    stream = torch.cuda.current_stream(device)
    if on_device:
        plan.run(frames, wdev, out, stream)
        if hout is not None:
            hout.copy_(out, non_blocking=True)
    else:
        # page-locked frames with 16-byte aligned rows are read in place: no device copy of the stack
        in_place = (isinstance(host, torch.Tensor) and host.is_pinned() and host.data_ptr() % 16 == 0
                    and (host.shape[-1] * host.element_size()) % 16 == 0)
        done = False
        if in_place:
            try:
                plan.run_from_host(host, None, wdev, out, hout, stream)
                done = True
            except _lib.FddmError as e:  # e.g. FDDM_B200_ZERO_COPY=0: nothing was queued, upload instead
                if e.code != _lib.FDDM_ERR_INVALID:
                    raise
        if not done:
            staging = torch.empty(_host_nbytes(host), dtype=torch.uint8, device=device)
            plan.run_from_host(host, staging, wdev, out, hout, stream)
    if hout is not None:
        stream.synchronize()  # the host arrays must outlive the queued copies
        return out, hout
    stream.synchronize()
    return out


def to_host(out: "torch.Tensor") -> np.ndarray:
    """Device result -> numpy array, through page-locked memory (the array keeps it alive)."""
    host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
    host.copy_(out)
    return host.numpy()


def ddm_fft_b200(img_seq, lags, nx, ny, nt, window, *, gpu_id: int = 0, precision: str = "ff", **kwargs) -> np.ndarray:
    """Image structure function, fft mode (Wiener-Khinchin), on the GB300."""
    _, hout = ddm_device(img_seq, lags, nx, ny, nt, window, mode="fft", precision=precision, gpu_id=gpu_id,
                         host_out=True)
    return hout.numpy()


def ddm_diff_b200(img_seq, lags, nx, ny, window, *, gpu_id: int = 0, precision: str = "ff", **kwargs) -> np.ndarray:
    """Image structure function, diff mode (direct differences), on the GB300."""
    _, hout = ddm_device(img_seq, lags, nx, ny, 0, window, mode="diff", precision=precision, gpu_id=gpu_id,
                         host_out=True)
    return hout.numpy()
