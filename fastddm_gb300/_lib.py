"""ctypes binding of ``libfddm_b200.so`` (the C ABI in ``include/fddm_b200.h``).

Loading never falls back to anything: if the shared library is missing, every
GPU entry point raises.  Call :func:`fastddm_gb300._build.build` (or
``__graft_entry__.build()``) to compile it.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from ._build import LIB_PATH

FDDM_OK = 0
FDDM_ERR_INVALID = 1
FDDM_ERR_NOMEM = 2
FDDM_ERR_CUDA = 3
FDDM_ERR_UNSUPPORTED = 4

PREC = {"ff": 0, "f64": 1, "f32": 2}
MODE = {"fft": 0, "diff": 1}
# numpy dtype name -> FDDM dtype code (include/fddm_b200.h)
DTYPE_CODE = {
    "uint8": 0,
    "int16": 1,
    "uint16": 2,
    "int32": 3,
    "uint32": 4,
    "int64": 5,
    "uint64": 6,
    "float32": 7,
    "float64": 8,
}

class Job(ctypes.Structure):
    """``fddm_b200_job`` of include/fddm_b200.h."""

    _fields_ = [
        ("mode", ctypes.c_int),
        ("d_img_seq", ctypes.c_void_p),
        ("dtype", ctypes.c_int),
        ("length", ctypes.c_uint64),
        ("height", ctypes.c_uint64),
        ("width", ctypes.c_uint64),
        ("lags", ctypes.POINTER(ctypes.c_uint32)),
        ("nlags", ctypes.c_uint64),
        ("nx", ctypes.c_uint64),
        ("ny", ctypes.c_uint64),
        ("nt", ctypes.c_uint64),
        ("d_window", ctypes.c_void_p),
        ("d_out", ctypes.c_void_p),
    ]


# every symbol the header declares, with (restype, argtypes)
_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p
_SIGNATURES = {
    "fddm_b200_version": (ctypes.c_int, []),
    "fddm_b200_last_error": (ctypes.c_char_p, []),
    "fddm_b200_workspace_size": (
        ctypes.c_int,
        [ctypes.c_int, ctypes.c_int, _u64, _u64, _u64, _u64, _u64, _u64, _u64, ctypes.c_int,
         ctypes.POINTER(ctypes.c_size_t)],
    ),
    "fddm_b200_ddm_fft": (
        ctypes.c_int,
        [_vp, ctypes.c_int, _u64, _u64, _u64, ctypes.POINTER(ctypes.c_uint32), _u64, _u64, _u64, _u64,
         _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int, _vp],
    ),
    "fddm_b200_ddm_diff": (
        ctypes.c_int,
        [_vp, ctypes.c_int, _u64, _u64, _u64, ctypes.POINTER(ctypes.c_uint32), _u64, _u64, _u64,
         _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int, _vp],
    ),
    "fddm_b200_ddm_from_host": (
        ctypes.c_int,
        [ctypes.c_int, _vp, ctypes.c_int, _u64, _u64, _u64, ctypes.POINTER(ctypes.c_uint32), _u64, _u64, _u64,
         _u64, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int, _vp],
    ),
    "fddm_b200_ddm_fft_noalloc": (
        ctypes.c_int,
        [_vp, ctypes.c_int, _u64, _u64, _u64, ctypes.POINTER(ctypes.c_uint32), _u64, _u64, _u64, _u64,
         _vp, _vp, ctypes.c_int, _vp],
    ),
    "fddm_b200_batch_workspace_size": (
        ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    ),
    "fddm_b200_batch_run": (
        ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_uint64, ctypes.c_int, _vp, ctypes.c_size_t, _vp]
    ),
    "fddm_b200_batch_create": (
        ctypes.c_int,
        [ctypes.POINTER(Job), ctypes.c_uint64, ctypes.c_int, _vp, ctypes.c_size_t, _vp, ctypes.POINTER(_vp)],
    ),
    "fddm_b200_batch_launch": (ctypes.c_int, [_vp, _vp]),
    "fddm_b200_batch_destroy": (ctypes.c_int, [_vp]),
    "fddm_b200_set_stage_timing": (ctypes.c_int, [ctypes.c_int]),
    "fddm_b200_stage_times": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "fddm_b200_launch_count": (ctypes.c_uint64, []),
    "fddm_b200_last_input_path": (ctypes.c_int, []),
    "fddm_b200_experiment_dft_stage": (ctypes.c_int, [ctypes.c_int, _vp, _u64, _vp, _vp]),
    "fddm_b200_set_autotune": (ctypes.c_int, [ctypes.c_int]),
    "fddm_b200_tuning_set": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _u64, _u64, ctypes.c_int, ctypes.c_int]),
    "fddm_b200_tuning_get": (
        ctypes.c_int,
        [ctypes.c_int, ctypes.c_int, _u64, _u64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    ),
    "fddm_b200_tuning_count": (ctypes.c_uint64, []),
    "fddm_b200_tuning_entry": (
        ctypes.c_int,
        [_u64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_u64),
         ctypes.POINTER(_u64), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    ),
    "fddm_b200_azimuthal_average": (
        ctypes.c_int,
        [_vp, _u64, _u64, _vp, _vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp],
    ),
    "fddm_b200_azimuthal_average_fast": (
        ctypes.c_int,
        [_vp, _u64, _u64, _vp, _vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp],
    ),
    "fddm_b200_polyfit_noise": (
        ctypes.c_int, [_vp, _u64, _u64, _vp, _vp, _u64, ctypes.c_double, _vp, _vp, _vp]
    ),
    "fddm_b200_fit_model_nparams": (ctypes.c_int, [ctypes.c_int]),
    "fddm_b200_fit_workspace_bytes": (ctypes.c_int, [ctypes.c_int, _u64, _u64, ctypes.POINTER(_u64)]),
    "fddm_b200_fit_lm": (
        ctypes.c_int,
        # model, m, x, ldx, nx, y, ldy, ny, w, ldw, nw, problems, nproblems, chain offsets, chain problems,
        # nchains, nvary, init, min, max, options, values, stderr, chisqr, nfev, info, status, residual,
        # covar, workspace, workspace bytes, stream
        [ctypes.c_int, _u64, _vp, _u64, _u64, _vp, _u64, _u64, _vp, _u64, _u64, _vp, _u64, _vp, _vp, _u64,
         ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u64, _vp],
    ),
    "fddm_b200_tiff_info": (
        ctypes.c_int,
        [ctypes.c_char_p, ctypes.POINTER(_u64), ctypes.POINTER(_u64), ctypes.POINTER(_u64),
         ctypes.POINTER(ctypes.c_int)],
    ),
    "fddm_b200_tiff_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_u64), _u64, _vp, ctypes.c_int]),
    "fddm_b200_sf_write": (
        ctypes.c_int,
        [ctypes.c_char_p, _vp, ctypes.c_int, _u64, _u64, _u64, _u64, _u64, _u64, _vp, _vp, _vp,
         ctypes.c_double, ctypes.c_double, _vp],
    ),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class FddmError(RuntimeError):
    """A call into the GB300 library returned an error status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"fddm_b200 error {code}: {msg}")
        self.code = code


def load(path: str | Path | None = None) -> ctypes.CDLL:
    """Load (once) and return the library with typed signatures."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p.name} is not built: the b200 core has no CPU fallback; "
                "run fastddm_gb300._build.build() first"
            )
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def check(code: int) -> None:
    """Raise :class:`FddmError` (MemoryError-like for FDDM_ERR_NOMEM) on a non-zero status."""
    if code == FDDM_OK:
        return
    msg = load().fddm_b200_last_error().decode(errors="replace")
    if code == FDDM_ERR_NOMEM:
        raise FddmError(code, "Not enough memory: " + msg)
    raise FddmError(code, msg)
