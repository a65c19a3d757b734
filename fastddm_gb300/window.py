"""Separable window functions applied to the frames before the spatial FFT.

Same definitions as ``src/python/window.py:54-161`` of the reference: the
periodic cosine-sum windows w(x) = sum_j (-1)^j a_j cos(2 pi j x / N) on
x = 0..N-1, combined as W(x, y) = w(x) w(y).  The terms are accumulated in the
same order and with the same expressions so the arrays are bit-identical.
"""

from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np

from ._config import DTYPE

_BLACKMAN = (7938 / 18608, 9240 / 18608, 1430 / 18608)
_BLACKMAN_HARRIS = (0.3635819, 0.4891775, 0.1365995, 0.0106411)


def _cosine_sum(n: int, coeffs: Sequence[float]) -> np.ndarray:
    x = np.linspace(0, (n - 1) / n, num=n)
    w = np.zeros(n)
    for j, a in enumerate(coeffs):
        w += (-1) ** j * a * np.cos(2.0 * np.pi * j * x)
    return w


def _separable(shape: Tuple[int, ...], coeffs: Sequence[float]) -> np.ndarray:
    *_, ydim, xdim = shape
    wx = _cosine_sum(xdim, coeffs)
    wy = _cosine_sum(ydim, coeffs)
    gx, gy = np.meshgrid(wx, wy)
    return (gx * gy).astype(DTYPE)


def blackman(shape: Tuple[int, ...]) -> np.ndarray:
    """Exact three-term Blackman window for an image (or sequence) shape."""
    return _separable(shape, _BLACKMAN)


def blackman_harris(shape: Tuple[int, ...]) -> np.ndarray:
    """Four-term Blackman-Harris window for an image (or sequence) shape."""
    return _separable(shape, _BLACKMAN_HARRIS)
