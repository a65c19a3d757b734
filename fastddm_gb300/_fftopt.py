"""Padded FFT lengths (``next_fast_len``) per backend core.

Restates ``src/python/_fftopt.py:29-150`` of the reference:

* ``'py'``   -> ``scipy.fft.next_fast_len``;
* ``'cpp'``  -> the smallest 2^a 3^b 5^c 7^d m >= target with m in {1, 11, 13};
* ``'cuda'`` -> the smallest 2^a 3^b 5^c 7^d >= target (optionally even);
* ``'b200'`` -> the ``'cpp'`` rule, so that nx, ny and therefore kx, ky and the
  1/sqrt(nx*ny) normalisation are identical to the ``cpp`` core; the kernels
  support every prime factor that rule can produce.

A power of two is always returned unchanged; unknown cores raise ``ValueError``.
"""

from __future__ import annotations

from scipy import fft as _scipy_fft


def next_power_of_2(target: int) -> int:
    """Smallest power of two >= ``target``."""
    return 1 << (target - 1).bit_length()


def _smallest_smooth(target: int, multipliers: tuple[int, ...], even: bool) -> int:
    best = next_power_of_2(target)
    odd_parts = []
    p3 = 1
    while p3 <= best:
        p5 = p3
        while p5 <= best:
            p7 = p5
            while p7 <= best:
                for m in multipliers:
                    if p7 * m <= best:
                        odd_parts.append(p7 * m)
                p7 *= 7
            p5 *= 5
        p3 *= 3
    for odd in odd_parts:
        v = odd * (2 if even else 1)
        while v < target:
            v *= 2
        if v < best:
            best = v
    return best


def next_fast_len(target: int, core: str = "b200", force_even: bool = False) -> int:
    """Next fast FFT length >= ``target`` for the given backend ``core``."""
    max_val = next_power_of_2(target)
    if target == max_val:
        return max_val
    c = core.upper()
    if c == "PY":
        return _scipy_fft.next_fast_len(target)
    if c in ("CPP", "B200"):
        return _smallest_smooth(target, (1, 11, 13), even=False)
    if c == "CUDA":
        return _smallest_smooth(target, (1,), even=force_even)
    raise ValueError("Mode not supported in `next_fast_len`.")
