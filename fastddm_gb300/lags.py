"""Lag (delay) helpers, same values as ``src/python/lags.py:38-152`` of the reference."""

from __future__ import annotations

import numpy as np


def logspace_int(stop: int, num: int = 50, endpoint: bool = False) -> np.ndarray:
    """``num`` quasi log-spaced integers in [1, stop] (``stop`` excluded unless ``endpoint``).

    Consecutive samples grow by a constant ratio; whenever the ratio would give
    a step below one, the sample is forced one above its predecessor and the
    ratio is recomputed for the remaining samples.  Samples are rounded at the end.
    """
    n_total = num if endpoint else num + 1
    ratio = stop ** (1.0 / n_total)
    out = np.empty(num)
    out[0] = 1
    for i in range(1, num):
        nxt = out[i - 1] * ratio
        if nxt - out[i - 1] >= 1.0:
            out[i] = nxt
        else:
            out[i] = out[i - 1] + 1
            ratio = (stop / out[i]) ** (1 / (n_total - i - 1))
    return np.round(out).astype(int)


def fibonacci(stop: int, endpoint: bool = False) -> np.ndarray:
    """Fibonacci numbers 1, 2, 3, 5, ... up to ``stop`` (excluded unless ``endpoint``)."""
    limit = stop if endpoint else stop - 1
    seq = [1, 2]
    while seq[-2] + seq[-1] <= limit:
        seq.append(seq[-2] + seq[-1])
    return np.array(seq, dtype=int)
