"""ORACLE - test infrastructure only; never part of the product path.

CPU restatement, in FP64 numpy, of FastDDM's ``cpp`` core for the
image-structure-function path.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import this module, and only as
the checker / the timed CPU baseline.

The reference ``cpp`` core (``src/cpp/ddm.cc`` + FFTW 3.3.10) cannot be built
here by the allowed routes: FFTW needs its own CMake build and a generated
``config.h``.  This restatement follows the reference's arithmetic step by
step and uses numpy's FP64 FFT in place of FFTW (both compute the DFT to FP64
rounding).  It is pinned against golden vectors produced by the reference's own
Python core (``tests/golden/make_golden.py``), which agrees with the ``cpp``
core to ~1e-11 in the reference's own cross-core tests.
"""

from __future__ import annotations

import math
from typing import Iterable, Optional, Sequence

import numpy as np


# ---------------------------------------------------------------------------
# spatial stage: src/cpp/ddm.cc:277-323 (copy into padded r2c rows, window,
# fftw r2c over (ny, nx), divide by sqrt(nx*ny))
# ---------------------------------------------------------------------------
def spatial_fft(img_seq: np.ndarray, nx: int, ny: int, window: Optional[np.ndarray] = None) -> np.ndarray:
    """Normalised half-plane spectrum F(t, ky, kx), complex128, ky unshifted."""
    T, H, W = img_seq.shape
    buf = np.zeros((T, ny, nx), dtype=np.float64)
    buf[:, :H, :W] = img_seq.astype(np.float64)
    if window is not None and np.size(window) > 0:
        buf[:, :H, :W] *= window  # ddm.cc:300-312
    F = np.fft.rfft2(buf, axes=(1, 2))
    return F / math.sqrt(float(nx * ny))  # ddm.cc:319-323


def shift_y(out: np.ndarray) -> np.ndarray:
    """y-fftshift of (rows, ny, nkx): make_shifted_isf, src/cpp/helper_ddm.cc:41-103."""
    return np.fft.fftshift(out, axes=1)


# ---------------------------------------------------------------------------
# fft mode: src/cpp/ddm.cc:325-446
# ---------------------------------------------------------------------------
def temporal_fft(Fq: np.ndarray, lags: Sequence[int], nt: int) -> np.ndarray:
    """(T, nq) spectrum columns -> (L + 2, nq): D per lag, PS, VAR (fft mode)."""
    T = Fq.shape[0]
    lags = [int(l) for l in lags]
    # ddm.cc:348-361 gather, /sqrt(nt), zero-pad to nt; :364 forward FFT
    X = np.fft.fft(Fq / math.sqrt(float(nt)), n=nt, axis=0)
    P = X.real * X.real + X.imag * X.imag  # :367-373
    tmp_avg = P[0] * float(nt) / float(T * T)  # :376-383
    Y = np.fft.fft(P, axis=0)  # :386, forward transform used as the inverse on real data
    # :389-414  tmp += |F(t)|^2 ; tmp += |F(T-1-t)|^2, walked t ascending
    sq = Fq.real * Fq.real + Fq.imag * Fq.imag
    inter = np.empty((2 * T,) + sq.shape[1:])
    inter[0::2] = sq
    inter[1::2] = sq[::-1]
    tmp = np.cumsum(inter, axis=0)[1::2]  # tmp after step t
    out = np.empty((len(lags) + 2,) + Fq.shape[1:])
    for i, lag in enumerate(lags):
        t = T - 1 - lag
        out[i] = (tmp[t] - 2.0 * Y[lag].real) / float(T - lag)
    ps = 0.5 * tmp[T - 1] / float(T)  # :423
    out[-2] = ps
    out[-1] = ps - tmp_avg  # :424
    return out


def ddm_fft(img_seq: np.ndarray, lags: Iterable[int], nx: int, ny: int, nt: int,
            window: Optional[np.ndarray] = None) -> np.ndarray:
    """ddm_fft<T> (src/cpp/ddm.cc:250-453): (L + 2, ny, nx//2 + 1) float64, y-shifted."""
    lags = list(lags)
    F = spatial_fft(img_seq, nx, ny, window)
    T = F.shape[0]
    Fq = F.reshape(T, -1)
    out = temporal_fft(Fq, lags, nt)
    return shift_y(out.reshape(len(lags) + 2, ny, nx // 2 + 1))


# ---------------------------------------------------------------------------
# diff mode: src/cpp/ddm.cc:37-192
# ---------------------------------------------------------------------------
def temporal_diff(Fq: np.ndarray, lags: Sequence[int]) -> np.ndarray:
    T = Fq.shape[0]
    out = np.empty((len(lags) + 2,) + Fq.shape[1:])
    for i, lag in enumerate(lags):  # :118-146
        lag = int(lag)
        d = Fq[lag:] - Fq[: T - lag]
        out[i] = (d.real * d.real + d.imag * d.imag).sum(axis=0) / float(T - lag)
    ps = (Fq.real * Fq.real + Fq.imag * Fq.imag).sum(axis=0) / float(T)  # :149-157
    re = Fq.real.sum(axis=0) / float(T)
    im = Fq.imag.sum(axis=0) / float(T)
    out[-2] = ps
    out[-1] = ps - re * re - im * im  # :160-164
    return out


def ddm_diff(img_seq: np.ndarray, lags: Iterable[int], nx: int, ny: int,
             window: Optional[np.ndarray] = None) -> np.ndarray:
    """ddm_diff<T> (src/cpp/ddm.cc:37-192): (L + 2, ny, nx//2 + 1) float64, y-shifted."""
    lags = list(lags)
    F = spatial_fft(img_seq, nx, ny, window)
    T = F.shape[0]
    out = temporal_diff(F.reshape(T, -1), lags)
    return shift_y(out.reshape(len(lags) + 2, ny, nx // 2 + 1))


# ---------------------------------------------------------------------------
# accuracy reference: the same quantities without cancellation
# ---------------------------------------------------------------------------
def ddm_exact(img_seq: np.ndarray, lags: Iterable[int], nx: int, ny: int,
              window: Optional[np.ndarray] = None) -> np.ndarray:
    """D, PS and VAR in extended precision (numpy long double where its FFT supports it).

    D(lag) = <|F(t+lag) - F(t)|^2>_t by direct differences (the diff-mode
    definition, src/cpp/ddm.cc:118-146), PS = <|F|^2>_t, VAR = <|F - <F>_t|^2>_t
    (the variance the reference computes as PS - |<F>|^2, ddm.cc:149-164).  Both
    reference algorithms lose digits to cancellation where D or VAR is small
    next to PS (fft mode: S1 + S2 - 2 Re C; VAR: PS - |<F>|^2); this one does
    not, so it is the yardstick for the error of every algorithm.
    """
    lags = [int(l) for l in lags]
    T, H, W = img_seq.shape
    ld = np.longdouble
    try:
        probe = np.fft.rfft2(np.ones((2, 2), dtype=ld))
        ext = probe.dtype.itemsize > 16
    except TypeError:  # pragma: no cover - numpy without long double FFTs
        ext = False
    dt = ld if ext else np.float64
    buf = np.zeros((T, ny, nx), dtype=dt)
    buf[:, :H, :W] = img_seq.astype(dt)
    if window is not None and np.size(window) > 0:
        buf[:, :H, :W] *= np.asarray(window).astype(dt)
    F = np.fft.rfft2(buf, axes=(1, 2)) / np.sqrt(dt(nx * ny))
    Fq = F.reshape(T, -1)
    out = np.empty((len(lags) + 2, Fq.shape[1]), dtype=dt)
    for i, lag in enumerate(lags):
        d = Fq[lag:] - Fq[: T - lag]
        out[i] = (d.real * d.real + d.imag * d.imag).sum(axis=0) / dt(T - lag)
    out[-2] = (Fq.real * Fq.real + Fq.imag * Fq.imag).sum(axis=0) / dt(T)
    G = Fq - Fq.sum(axis=0) / dt(T)
    out[-1] = (G.real * G.real + G.imag * G.imag).sum(axis=0) / dt(T)
    return shift_y(out.reshape(len(lags) + 2, ny, nx // 2 + 1)).astype(np.float64)


def sampled_exact(img_seq: np.ndarray, lags: Iterable[int], nx: int, ny: int, cols: Sequence[int],
                  window: Optional[np.ndarray] = None, threads: int = 8) -> np.ndarray:
    """D, PS and VAR at the kx columns `cols` (every ky), without cancellation, for large stacks.

    The spectrum of the sampled columns comes from direct FP64 DFTs of every
    frame (rows against exp(-2 pi i x kx / nx), then columns against
    exp(-2 pi i y ky / ny), scaled by 1/sqrt(nx ny) as ddm.cc:319-323 does);
    D(lag) by direct differences (src/cpp/ddm.cc:118-146), PS = <|F|^2>_t and
    VAR = <|F - <F>_t|^2>_t.  Returns (L + 2, ny, len(cols)), y-fftshifted like
    the full result's columns `cols`.  Its own error is ~1e-16 sqrt(PS / D).
    """
    from concurrent.futures import ThreadPoolExecutor

    lags = [int(l) for l in lags]
    T, H, W = img_seq.shape
    C = len(cols)
    ex = np.exp(-2j * np.pi * np.outer(np.arange(W), np.asarray(cols)) / nx)
    exr = np.ascontiguousarray(np.concatenate([ex.real, ex.imag], axis=1))  # (W, 2C)
    ey = np.exp(-2j * np.pi * np.outer(np.arange(ny), np.arange(H)) / ny)   # (ny, H), natural ky order
    win = None if window is None or np.size(window) == 0 else np.asarray(window, dtype=np.float64)
    F = np.empty((T, ny, C), dtype=np.complex128)
    for t0 in range(0, T, 16):
        blk = np.asarray(img_seq[t0:t0 + 16]).astype(np.float64)
        if win is not None:
            blk *= win
        a = blk @ exr
        F[t0:t0 + 16] = np.einsum("yh,thc->tyc", ey, a[..., :C] + 1j * a[..., C:], optimize=True)
    F /= math.sqrt(float(nx * ny))
    Fq = F.reshape(T, ny * C)

    def chunk(c0):
        f = Fq[:, c0:c0 + 256]
        o = np.empty((len(lags) + 2, f.shape[1]))
        for i, lag in enumerate(lags):
            d = f[lag:] - f[: T - lag]
            o[i] = (d.real * d.real + d.imag * d.imag).sum(axis=0) / float(T - lag)
        o[-2] = (f.real * f.real + f.imag * f.imag).sum(axis=0) / float(T)
        g = f - f.mean(axis=0)
        o[-1] = (g.real * g.real + g.imag * g.imag).sum(axis=0) / float(T)
        return o

    with ThreadPoolExecutor(max_workers=threads) as ex_:
        parts = list(ex_.map(chunk, range(0, ny * C, 256)))
    out = np.concatenate(parts, axis=1).reshape(len(lags) + 2, ny, C)
    return np.fft.fftshift(out, axes=1)


# ---------------------------------------------------------------------------
# front door pieces: src/python/_ddm.py:128-198, _fftopt.py:29-150
# ---------------------------------------------------------------------------
def next_fast_len_cpp(target: int) -> int:
    """Smallest 2^a 3^b 5^c 7^d m >= target, m in {1, 11, 13}; powers of 2 unchanged."""
    p2 = 1 << (target - 1).bit_length()
    if p2 == target:
        return target
    best = p2
    for m in (1, 11, 13):
        a = 1
        while a * m <= best:
            b = a
            while b * m <= best:
                c = b
                while c * m <= best:
                    v = c * m
                    while v < target:
                        v *= 2
                    best = min(best, v)
                    c *= 7
                b *= 5
            a *= 3
    return best


def axes(nx: int, ny: int):
    """kx, ky of the result (src/python/_ddm.py:190-191)."""
    kx = 2 * np.pi * np.fft.fftfreq(nx)[: nx // 2 + 1]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(ny))
    return kx, ky


def prepare_lags(lags: Iterable[int], length: int) -> np.ndarray:
    """Sorted unique lags with 0 dropped (src/python/_ddm.py:139-159)."""
    lags = np.array(sorted(set(lags)))
    if lags.size and lags[0] == 0:
        lags = lags[1:]
    return lags


# ---------------------------------------------------------------------------
# azimuthal average: src/python/azimuthalaverage.py:277-478 (loops kept, small inputs)
# ---------------------------------------------------------------------------
def azimuthal_average_array(data: np.ndarray, dist: np.ndarray, bins, rng, mask, weights, counts,
                            eval_err: bool = True):
    """Loop restatement of azimuthal_average_array; returns (avg, err, x, bin_edges)."""
    m = np.full(dist.shape, True) if mask is None else mask.astype(bool).copy()
    counts = np.ones(dist.shape) if counts is None else counts
    if rng is None:
        x_min, x_max = np.min(dist), np.max(dist)
    else:
        x_min, x_max = rng
        if x_min > x_max:
            x_min, x_max = x_max, x_min
    if isinstance(bins, int):
        edges = np.linspace(x_min, x_max, bins, dtype=np.float64)
        n_bins = bins
    else:
        edges = np.array(bins).astype(np.float64)
        n_bins = len(bins)
        x_min = bins[0]
    idx = np.searchsorted(edges, dist)
    m[(idx == n_bins) | (dist < x_min)] = False
    wi = counts.astype(np.float64)
    wi2 = counts.astype(np.float64)
    if weights is not None:
        wi = wi * weights
        wi2 = wi2 * weights ** 2
    m[np.logical_not(wi)] = False
    x = np.zeros(n_bins)
    avg = np.zeros((n_bins, len(data)))
    err = np.zeros((n_bins, len(data)))
    sw = np.zeros(n_bins)
    sw2 = np.zeros(n_bins)
    ny, nx = dist.shape
    for i in range(ny):
        for j in range(nx):
            if m[i, j]:
                sw[idx[i, j]] += wi[i, j]
                sw2[idx[i, j]] += wi2[i, j]
    for i in range(ny):
        for j in range(nx):
            if m[i, j]:
                b = idx[i, j]
                x[b] += dist[i, j] * wi[i, j] / sw[b]
                avg[b] += data[:, i, j] * wi[i, j] / sw[b]
    avg[sw == 0] = np.nan
    for b in range(n_bins):
        if sw[b] == 0:
            x[b] = 0.5 * (edges[b - 1] + edges[b]) if b > 0 else edges[0]
    if eval_err:
        bias = [s - (s2 / s) if s > 0 else 0 for s, s2 in zip(sw, sw2)]
        with np.errstate(divide="ignore", invalid="ignore"):
            for i in range(ny):
                for j in range(nx):
                    if m[i, j]:
                        b = idx[i, j]
                        err[b] += wi[i, j] * (data[:, i, j] - avg[b]) ** 2 / bias[b]
        err[sw == 0] = np.nan
        np.sqrt(err, out=err)
    else:
        err = None
    return avg, err, x, edges


def azimuthal_average(data: np.ndarray, kx: np.ndarray, ky: np.ndarray, width: int, bins, rng=None,
                      mask=None, weights=None, eval_err: bool = True):
    """azimuthal_average (src/python/azimuthalaverage.py:481-564) on a (rows, ny, nkx) array."""
    counts = np.full(data.shape[1:], 2)
    counts[:, 0] = 1
    counts[:, -1] = 1 if width % 2 == 0 else 2
    X, Y = np.meshgrid(kx, ky)
    dist = np.sqrt(X ** 2 + Y ** 2)
    return azimuthal_average_array(data, dist, bins, rng, mask, weights, counts, eval_err)


# ---------------------------------------------------------------------------
# error metrics used by the tests and the bench report
# ---------------------------------------------------------------------------
def rel_err(test: np.ndarray, ref: np.ndarray, skip_dc: bool = False, ny: Optional[int] = None,
            floor: float = 0.0) -> float:
    """Max elementwise |test - ref| / |ref| over the structure-function rows.

    With ``skip_dc`` the q = 0 mode (row ny//2, column 0 after the y shift) is
    excluded.  ``floor`` > 0 measures entries smaller than ``floor`` times the
    largest |ref| of their row against that threshold instead (for values that
    are exactly zero in exact arithmetic).
    """
    t = np.asarray(test, dtype=np.float64)
    r = np.asarray(ref, dtype=np.float64)
    den = np.abs(r)
    if floor > 0 and r.ndim >= 2:
        rowmax = np.max(np.abs(r).reshape(r.shape[0], -1), axis=1).reshape((-1,) + (1,) * (r.ndim - 1))
        den = np.maximum(den, floor * rowmax)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = np.abs(t - r) / den
    e = np.where(den == 0, np.where(t == r, 0.0, np.inf), e)
    if skip_dc:
        ny = ny if ny is not None else r.shape[-2]
        e = e.copy()
        e[..., ny // 2, 0] = 0.0
    return float(np.max(e)) if e.size else 0.0
