"""Camera-noise (B) estimates from an image structure function or its
azimuthal average: interface and results of the reference's
``src/python/noise_est.py`` (``estimate_camera_noise`` ``:759-841``).

Modes: "zero", "min", "high_q", "power_spec", "var", "polyfit".  Everything
but "polyfit" on an ``ImageStructureFunction`` is a reduction over at most a
few hundred thousand values and is done with numpy exactly as the reference
does.  "polyfit" on an ``ImageStructureFunction`` is the reference's Python
loop of ``numpy.polyfit`` calls, one per (ky, kx) pixel (525k fits for a
1024 x 1024 stack); here it is one device kernel (``fddm_b200_polyfit_noise``)
applying the fit's least-squares operator, which is the same for every pixel,
to the device copy of the data.
"""

from __future__ import annotations

import ctypes
import warnings
from typing import Optional, Tuple, Union

import numpy as np

from . import _lib
from ._config import DTYPE
from .azimuthalaverage import AzimuthalAverage
from .imagestructurefunction import ImageStructureFunction

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _full(shape, value):
    return np.full(shape, fill_value=value, dtype=DTYPE)


def _swap_range(k_min: float, k_max: float) -> Tuple[float, float]:
    if k_min > k_max:
        k_min, k_max = k_max, k_min
        warnings.warn("Given k_min larger than k_max. Input values swapped.")
    return k_min, k_max


# ---------------------------------------------------------------------------
# AzimuthalAverage (src/python/noise_est.py:75-379)
# ---------------------------------------------------------------------------
def _aa_zero(obj: AzimuthalAverage):
    n = len(obj.k)
    return np.zeros(n, dtype=DTYPE), np.zeros(n, dtype=DTYPE)


def _aa_min(obj: AzimuthalAverage):
    i = np.nanargmin(obj.data[:, 0])
    value = obj.data[i, 0]
    unc = value if obj.err is None else obj.err[i, 0]
    return _full(len(obj.k), value), _full(len(obj.k), unc)


def _aa_range(obj: AzimuthalAverage, k_min, k_max):
    k_min = np.max(obj.k) if k_min is None else k_min
    k_max = np.max(obj.k) if k_max is None else k_max
    k_min, k_max = _swap_range(k_min, k_max)
    return (obj.k >= k_min) & (obj.k <= k_max)


def _aa_mean(values: np.ndarray, errors: Optional[np.ndarray], factor: float, n: int):
    value = factor * np.nanmean(values)
    if errors is None:
        unc = value
    else:
        # the reference counts every selected entry (np.size of the NaN test), NaN or not
        numel = np.size(~np.isnan(errors))
        unc = factor * np.sqrt(np.nansum(errors ** 2)) / numel if numel > 0 else np.nan
    return _full(n, value), _full(n, unc)


def _aa_high_q(obj: AzimuthalAverage, k_min=None, k_max=None):
    m = _aa_range(obj, k_min, k_max)
    return _aa_mean(obj.data[m], None if obj.err is None else obj.err[m], 1, len(obj.k))


def _aa_power_spec(obj: AzimuthalAverage, k_min=None, k_max=None):
    m = _aa_range(obj, k_min, k_max)
    e = obj.power_spec_err
    return _aa_mean(obj.power_spec[m], None if e is None else e[m], 2, len(obj.k))


def _aa_var(obj: AzimuthalAverage, k_min=None, k_max=None):
    m = _aa_range(obj, k_min, k_max)
    e = obj.var_err
    return _aa_mean(obj.var[m], None if e is None else e[m], 2, len(obj.k))


def _aa_polyfit(obj: AzimuthalAverage, num_points: int = 5):
    deg = 2
    num_points = max(deg + 1, num_points)
    noise, unc = _aa_zero(obj)
    x = obj.tau[:num_points]
    for i in range(len(obj.k)):
        if np.isnan(obj.data[i, 0]):
            noise[i] = np.nan
            unc[i] = np.nan
            continue
        y = obj.data[i, :num_points]
        w = None
        if obj.err is not None and not np.any(np.isnan(obj.err[i, :num_points])):
            w = 1 / obj.err[i, :num_points]
        p, pcov = np.polyfit(x, y, deg=deg, w=w, cov="unscaled")
        noise[i] = p[-1]
        unc[i] = np.sqrt(np.diag(pcov))[-1]
    return noise, unc


# ---------------------------------------------------------------------------
# ImageStructureFunction (src/python/noise_est.py:382-756)
# ---------------------------------------------------------------------------
def _mask(obj: ImageStructureFunction, mask):
    _, ny, nx = obj.shape
    if mask is None:
        return np.full((ny, nx), True)
    if mask.dtype != bool:
        warnings.warn("Given mask not of boolean type. Casting to bool.")
        return mask.astype(bool)
    return mask


def _sf_zero(obj: ImageStructureFunction):
    _, ny, nx = obj.shape
    return np.zeros((ny, nx), dtype=DTYPE), np.zeros((ny, nx), dtype=DTYPE)


def _sf_min(obj: ImageStructureFunction, mask=None):
    _, ny, nx = obj.shape
    mask = _mask(obj, mask)
    # the reference maps the index into the masked values back as if it were an
    # index into the full plane (identical when nothing is masked)
    i = np.nanargmin(obj.data[0, mask])
    value = obj.data[0, i // nx, i % nx]
    return _full((ny, nx), value), _full((ny, nx), value)


def _sf_range(obj: ImageStructureFunction, k_min, k_max, mask):
    kmax = max(np.max(obj.kx), np.max(obj.ky))
    k_min = kmax if k_min is None else k_min
    k_max = kmax if k_max is None else k_max
    k_min, k_max = _swap_range(k_min, k_max)
    mask = _mask(obj, mask)
    kx, ky = np.meshgrid(obj.kx, obj.ky)
    k = np.sqrt(kx ** 2 + ky ** 2)
    return (k >= k_min) & (k <= k_max) & mask


def _sf_high_q(obj: ImageStructureFunction, k_min=None, k_max=None, mask=None):
    m = _sf_range(obj, k_min, k_max, mask)
    value = np.nanmean(obj.data[:, m])
    return _full(obj.shape[1:], value), _full(obj.shape[1:], value)


def _sf_power_spec(obj: ImageStructureFunction, k_min=None, k_max=None, mask=None):
    m = _sf_range(obj, k_min, k_max, mask)
    value = 2 * np.nanmean(obj.power_spec[m])
    return _full(obj.shape[1:], value), _full(obj.shape[1:], value)


def _sf_var(obj: ImageStructureFunction, k_min=None, k_max=None, mask=None):
    m = _sf_range(obj, k_min, k_max, mask)
    value = 2 * np.nanmean(obj.var[m])
    return _full(obj.shape[1:], value), _full(obj.shape[1:], value)


def polyfit_operator(x: np.ndarray) -> Tuple[np.ndarray, float]:
    """(3, n) least-squares operator of the quadratic fit on abscissae `x` and
    the (2, 2) entry of the unscaled covariance, from the column-scaled
    Vandermonde system that numpy.polyfit solves."""
    v = np.vander(np.asarray(x, dtype=np.float64), 3)
    scale = np.sqrt((v * v).sum(axis=0))
    vs = v / scale
    op = np.linalg.pinv(vs) / scale[:, None]
    vbase = np.linalg.inv(vs.T @ vs) / np.outer(scale, scale)
    return np.ascontiguousarray(op), float(vbase[2, 2])


def _sf_polyfit(obj: ImageStructureFunction, num_points: int = 5):
    deg = 2
    num_points = max(deg + 1, num_points)
    x = np.asarray(obj.tau[:num_points], dtype=np.float64)
    n = len(x)
    if n <= deg + 1:
        raise ValueError("the number of data points must exceed order to scale the covariance matrix")
    op, cov22 = polyfit_operator(x)
    _, ny, nx = obj.shape
    q = ny * nx
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("the polyfit noise estimate runs on the GPU: no CUDA device available")
    dev = obj._device_data
    if dev is not None:
        rows = dev
        device = dev.device
    else:
        device = torch.device("cuda", 0)
        rows = torch.from_numpy(np.ascontiguousarray(obj._data[:n], dtype=np.float64)).to(device)
    noise = torch.empty(q, dtype=torch.float64, device=device)
    unc = torch.empty(q, dtype=torch.float64, device=device)
    lib = _lib.load()
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream(device)
        _lib.check(lib.fddm_b200_polyfit_noise(rows.data_ptr(), q, q, x.ctypes.data, op.ctypes.data, n, cov22,
                                               noise.data_ptr(), unc.data_ptr(), stream.cuda_stream))
        stream.synchronize()
    return noise.cpu().numpy().reshape(ny, nx).astype(DTYPE), unc.cpu().numpy().reshape(ny, nx).astype(DTYPE)


_AA = {"zero": _aa_zero, "min": _aa_min, "high_q": _aa_high_q, "power_spec": _aa_power_spec, "var": _aa_var,
       "polyfit": _aa_polyfit}
_SF = {"zero": _sf_zero, "min": _sf_min, "high_q": _sf_high_q, "power_spec": _sf_power_spec, "var": _sf_var,
       "polyfit": _sf_polyfit}


def estimate_camera_noise(obj: Union[ImageStructureFunction, AzimuthalAverage], mode: str = "zero",
                          **kwargs) -> Tuple[np.ndarray, np.ndarray]:
    """Noise factor B and its uncertainty, per wavevector (``noise_est.py:759-841``).

    "high_q", "power_spec" and "var" take ``k_min`` / ``k_max`` (default: the
    largest k; swapped with a warning when reversed); for an
    ``ImageStructureFunction`` "min", "high_q", "power_spec" and "var" also
    take a boolean ``mask``; "polyfit" takes ``num_points`` (default 5).
    """
    if isinstance(obj, ImageStructureFunction):
        table = _SF
    elif isinstance(obj, AzimuthalAverage):
        table = _AA
    else:
        raise TypeError(f"Input type {type(obj)} not supported.")
    if mode not in table:
        raise RuntimeError(f"Unknown mode '{mode}' selected. Only possible options are {list(table.keys())}.")
    return table[mode](obj=obj, **kwargs)
