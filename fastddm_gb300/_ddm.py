r"""``ddm()``: differential dynamic microscopy front door with backend registry.

Mirrors ``src/python/_ddm.py:77-198`` of the reference: the same validation,
messages and argument assembly, and the same axes:

    D(q, dt)  = < |I~(q, t + dt) - I~(q, t)|^2 >_t
    PS(q)     = < |I~(q, t)|^2 >_t
    VAR(q)    = < |I~(q, t) - <I~(q)>_t|^2 >_t

with I~ the 2D FFT of a frame divided by sqrt(nx * ny).  The registry holds
the GB300 core ``'b200'``; the reference's ``_backend`` can register the same
two functions, ``ddm_fft_b200`` and ``ddm_diff_b200``, under that key.
"""

from __future__ import annotations

import warnings
from typing import Callable, Dict, Iterable, Optional

import numpy as np

from ._config import DTYPE
from ._ddm_b200 import ddm_device, ddm_diff_b200, ddm_fft_b200
from ._fftopt import next_fast_len
from .imagestructurefunction import ImageStructureFunction

_backend: Dict[str, Dict[str, Callable]] = {
    "b200": {
        "diff": ddm_diff_b200,
        "fft": ddm_fft_b200,
    }
}


def _prepare(img_seq, lags, core: str, mode: str, window):
    """The front door's checks and derived sizes (``src/python/_ddm.py:128-173``)."""
    cores = list(_backend.keys())
    modes = ["diff", "fft"]
    if core not in cores:
        raise RuntimeError(f"Unknown core '{core}' selected. Only possible options are {cores}.")
    if mode not in modes:
        raise RuntimeError(f"Unknown mode '{mode}' selected. Only possible options are {modes}.")

    lags = np.array(sorted(set(lags)))
    dim_t, dim_y, dim_x = img_seq.shape
    if np.min(lags) < 0:
        raise RuntimeError("Negative lags are not possible.")
    if np.max(lags) > dim_t - 1:
        raise RuntimeError(f"Lags larger than len(img_seq) - 1 = {dim_t - 1} are not possible.")
    if lags[0] == 0:
        warnings.warn("Found 0 in lags. Removed for compatibility with other functions.")
        lags = lags[1:]

    if window is None:
        window = np.array([], dtype=DTYPE)
    elif tuple(window.shape) != (dim_y, dim_x):
        raise RuntimeError(f"Window with shape {window.shape} incompatible with image shape {(dim_y, dim_x)}.")

    nx = next_fast_len(dim_x, core)
    ny = next_fast_len(dim_y, core)
    nt = next_fast_len(2 * dim_t, core) if mode == "fft" else 0

    kx = 2 * np.pi * np.fft.fftfreq(nx)[: (nx // 2 + 1)]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(ny))

    return lags, window, nx, ny, nt, kx, ky


def ddm(
    img_seq,
    lags: Iterable[int],
    *,
    core: str = "b200",
    mode: str = "fft",
    window: Optional[np.ndarray] = None,
    keep_on_device: bool = True,
    **kwargs,
) -> ImageStructureFunction:
    """Image structure function of ``img_seq`` (shape ``(t, y, x)``) at the given lags.

    Raises RuntimeError for an unknown core or mode, negative lags, lags beyond
    ``len(img_seq) - 1`` or a window whose shape differs from a frame's; lag 0
    is removed with a warning.  ``kwargs`` go to the backend (``gpu_id``,
    ``precision``).  With ``keep_on_device`` the returned object also holds the
    device copy of its data, used by ``azimuthal_average``.
    """
    backend = _backend
    lags, window, nx, ny, nt, kx, ky = _prepare(img_seq, lags, core, mode, window)

    if core == "b200" and keep_on_device:
        dev, host = ddm_device(img_seq, lags, nx, ny, nt, window, mode=mode, host_out=True, **kwargs)
        data = host.numpy()
    else:
        func = backend[core][mode]
        args = [img_seq, lags, nx, ny] + ([nt] if mode == "fft" else []) + [window.astype(DTYPE)]
        data, dev = func(*args, **kwargs), None
    return ImageStructureFunction(
        data, kx.astype(DTYPE), ky.astype(DTYPE), nx, ny, lags.astype(DTYPE), _device_data=dev
    )
