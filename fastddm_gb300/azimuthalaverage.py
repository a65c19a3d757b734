"""Azimuthal average of the image structure function on the GB300.

Interface of the reference's ``src/python/azimuthalaverage.py``:
``AzimuthalAverage`` (``:80-274``), ``azimuthal_average_array`` (``:277-478``)
and ``azimuthal_average`` (``:481-564``).

Work split:

* host (vectorised numpy, O(pixels)): argument checks, bin edges
  (``linspace`` edges, not ``bins + 1``), ``searchsorted`` bin indices, the mask
  (out-of-range, below ``x_min``, masked, zero weight), per-bin sums of weights
  and the weighted mean ``k`` per bin.  ``np.bincount`` adds in pixel order,
  the order of the reference's loops, so these match it bit for bit;
* device (``fddm_b200_azimuthal_average``, O(pixels x rows)): the weighted mean
  and unbiased weighted standard deviation of every row in every bin, one
  thread per (bin, row) summing in pixel order with the reference's operation
  order, so they also match the reference's loops bit for bit.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass
from typing import Iterable, Optional, Tuple, Union

import numpy as np

from . import _lib
from ._config import DTYPE
from .imagestructurefunction import ImageStructureFunction

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


@dataclass
class AzimuthalAverage:
    """Azimuthal average container (same fields as the reference)."""

    _data: np.ndarray
    _err: Optional[np.ndarray]
    k: np.ndarray
    tau: np.ndarray
    bin_edges: np.ndarray

    @property
    def data(self) -> np.ndarray:
        return self._data[:, :-2]

    @property
    def err(self) -> Optional[np.ndarray]:
        return None if self._err is None else self._err[:, :-2]

    @property
    def power_spec(self) -> np.ndarray:
        return self._data[:, -2]

    @property
    def var(self) -> np.ndarray:
        return self._data[:, -1]

    @property
    def power_spec_err(self) -> Optional[np.ndarray]:
        return None if self._err is None else self._err[:, -2]

    @property
    def var_err(self) -> Optional[np.ndarray]:
        return None if self._err is None else self._err[:, -1]

    def save(self, fname: str = "analysis_blob") -> None:
        """Write the object to ``fname`` (``.aa.ddm`` appended if missing) in the
        reference's file format (``azimuthalaverage.py:197-212``)."""
        from ._io import save_aa

        save_aa(self, fname)

    @property
    def shape(self) -> Tuple[int, int]:
        return self.data.shape


@dataclass
class BinSetup:
    """Host-side result of the binning set-up (``azimuthalaverage.py:349-432``)."""

    bin_edges: np.ndarray
    n_bins: int
    valid: np.ndarray      # flattened bool, pixel takes part
    bin_idx: np.ndarray    # flattened searchsorted index
    wi: np.ndarray         # flattened counts x weights
    sum_wi: np.ndarray
    sum_wi2: Optional[np.ndarray]
    k: np.ndarray


def bin_setup(dist: np.ndarray, bins, range, mask, weights, counts, eval_err: bool) -> BinSetup:
    """Validate the arguments and compute edges, indices, weights and per-bin sums."""
    if mask is not None:
        m = mask.copy()
        if mask.shape != dist.shape:
            raise ValueError("mask shape and dist shape must be the same.")
        if mask.dtype != bool:
            m = mask.astype(bool)
            warnings.warn("mask is not of boolean type, it is cast to bool.")
    else:
        m = np.full(dist.shape, True)
    if weights is not None:
        if weights.shape != dist.shape:
            raise ValueError("weights shape and dist shape must be the same.")
        if np.any(weights < 0):
            raise ValueError("weights must be non-negative.")
    if counts is not None:
        if counts.shape != dist.shape:
            raise ValueError("counts shape and dist shape must be the same.")
    else:
        counts = np.ones(dist.shape, dtype=DTYPE)

    if range is None:
        x_min, x_max = np.min(dist), np.max(dist)
    else:
        x_min, x_max = range
        if x_min > x_max:
            x_min, x_max = x_max, x_min

    if isinstance(bins, int):
        edges = np.linspace(x_min, x_max, bins, dtype=DTYPE)
        n_bins = bins
    elif isinstance(bins, Iterable):
        # the same (for lists: lexicographic) comparison the reference applies
        if not np.all(bins[1:] >= bins[:-1]):
            raise ValueError("bins must be monotonically increasing.")
        edges = np.array(bins).astype(DTYPE)
        n_bins = len(bins)
        x_min = bins[0]
    else:
        raise ValueError("bins must be an int or an iterable.")

    bin_idx = np.searchsorted(edges, dist)
    m[(bin_idx == n_bins) | (dist < x_min)] = False
    wi = counts.astype(DTYPE)
    if weights is not None:
        wi *= weights
    wi2 = None
    if eval_err:
        wi2 = counts.astype(DTYPE)
        if weights is not None:
            wi2 *= weights ** 2
    m[np.logical_not(wi)] = False

    valid = m.ravel()
    bidx = bin_idx.ravel()
    sel = bidx[valid]
    sum_wi = np.bincount(sel, weights=wi.ravel()[valid], minlength=n_bins).astype(DTYPE)[:n_bins]
    sum_wi2 = None
    if eval_err:
        sum_wi2 = np.bincount(sel, weights=wi2.ravel()[valid], minlength=n_bins).astype(DTYPE)[:n_bins]
    with np.errstate(divide="ignore", invalid="ignore"):
        terms = dist.ravel()[valid] * wi.ravel()[valid] / sum_wi[sel]
    k = np.bincount(sel, weights=terms, minlength=n_bins).astype(DTYPE)[:n_bins]
    for b in np.flatnonzero(sum_wi == 0):
        k[b] = 0.5 * (edges[b - 1] + edges[b]) if b > 0 else edges[0]
    return BinSetup(edges, n_bins, valid, bidx, wi.ravel(), sum_wi, sum_wi2, k)


def _device_of(gpu_id):
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("the b200 azimuthal average needs a CUDA device (GB300)")
    return torch.device("cuda", int(gpu_id))


def _run_device(data_dev, setup: BinSetup, eval_err: bool, device, exact: bool = True,
                host: bool = True):
    nrows = int(data_dev.shape[0])
    npix = int(np.prod(data_dev.shape[1:]))
    n_bins = setup.n_bins
    pix = np.flatnonzero(setup.valid).astype(np.int32)
    order = np.argsort(setup.bin_idx[pix], kind="stable")
    pix_sorted = np.ascontiguousarray(pix[order])
    cnt = np.bincount(setup.bin_idx[pix], minlength=n_bins)[:n_bins]
    offsets = np.zeros(n_bins + 1, dtype=np.int32)
    np.cumsum(cnt, out=offsets[1:])
    with np.errstate(divide="ignore", invalid="ignore"):
        bias = None
        if eval_err:
            bias = np.where(setup.sum_wi > 0, setup.sum_wi - setup.sum_wi2 / setup.sum_wi, 0.0).astype(DTYPE)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(device)

    d_off, d_pix, d_w, d_sw = dev(offsets), dev(pix_sorted if len(pix_sorted) else np.zeros(1, np.int32)), dev(setup.wi), dev(setup.sum_wi)
    d_bias = dev(bias) if eval_err else None
    avg = torch.empty((n_bins, nrows), dtype=torch.float64, device=device)
    err = torch.empty((n_bins, nrows), dtype=torch.float64, device=device) if eval_err else None
    lib = _lib.load()
    data_dev = data_dev.contiguous()
    fn = lib.fddm_b200_azimuthal_average if exact else lib.fddm_b200_azimuthal_average_fast
    with torch.cuda.device(device):
        code = fn(
            data_dev.data_ptr(), nrows, npix, d_off.data_ptr(), d_pix.data_ptr(), n_bins, d_w.data_ptr(),
            d_sw.data_ptr(), d_bias.data_ptr() if d_bias is not None else None, avg.data_ptr(),
            err.data_ptr() if err is not None else None, torch.cuda.current_stream(device).cuda_stream,
        )
    _lib.check(code)
    if not host:
        return avg, err
    return avg.cpu().numpy(), (err.cpu().numpy() if err is not None else None)


def azimuthal_average_array(
    data,
    dist: np.ndarray,
    bins: Optional[Union[int, Iterable[float]]] = 10,
    range: Optional[Tuple[float, float]] = None,
    mask: Optional[np.ndarray] = None,
    weights: Optional[np.ndarray] = None,
    counts: Optional[np.ndarray] = None,
    eval_err: Optional[bool] = True,
    *,
    gpu_id: int = 0,
    exact: bool = True,
) -> Tuple[np.ndarray, ...]:
    """Weighted azimuthal average of a 3D array (numpy, or a CUDA tensor already on the device).

    Returns ``(avg, err, k, bin_edges)``; ``avg``/``err`` have shape
    ``(n_bins, len(data))``, empty bins are NaN, ``err`` is None when
    ``eval_err`` is False.  ``exact=True`` reproduces the reference's per-pixel
    loops bit for bit; ``exact=False`` sums each bin with a warp of fused
    multiply-adds (rounding-level differences, much faster on large maps).
    """
    dim_y, dim_x = tuple(data.shape[-2:])
    if dist.shape != (dim_y, dim_x):
        raise ValueError("dist shape must be compatible with data shape.")
    setup = bin_setup(dist, bins, range, mask, weights, counts, bool(eval_err))
    device = _device_of(gpu_id)
    if torch is not None and isinstance(data, torch.Tensor):
        data_dev = data.to(device=device, dtype=torch.float64)
    else:
        data_dev = torch.from_numpy(np.ascontiguousarray(data, dtype=np.float64)).to(device)
    avg, err = _run_device(data_dev, setup, bool(eval_err), device, exact)
    return avg, err, setup.k, setup.bin_edges


def azimuthal_average(
    img_str_func: ImageStructureFunction,
    bins: Optional[Union[int, Iterable[float]]] = 10,
    range: Optional[Tuple[float, float]] = None,
    mask: Optional[np.ndarray] = None,
    weights: Optional[np.ndarray] = None,
    eval_err: Optional[bool] = True,
    *,
    gpu_id: int = 0,
    exact: bool = True,
) -> AzimuthalAverage:
    """Azimuthal average of an image structure function (reference ``:481-564``).

    ``exact`` as in :func:`azimuthal_average_array`.

    Column 0 counts once, the last column once when the full width is even,
    every other column twice (its mirror image in the full plane).
    """
    counts = np.full(img_str_func.shape[1:], 2)
    counts[:, 0] = 1
    counts[:, -1] = 1 if img_str_func.width % 2 == 0 else 2
    gx, gy = np.meshgrid(img_str_func.kx, img_str_func.ky)
    k_modulus = np.sqrt(gx ** 2 + gy ** 2)
    data = img_str_func._device_data if img_str_func._device_data is not None else img_str_func._data
    avg, err, k, edges = azimuthal_average_array(
        data, k_modulus, bins, range, mask, weights, counts, eval_err, gpu_id=gpu_id, exact=exact
    )
    return AzimuthalAverage(avg, err, k, img_str_func.tau, edges)
