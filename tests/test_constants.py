"""The literal DFT constants compiled into the kernels (csrc/dft_consts.cuh) against 60-digit values."""

import re
from pathlib import Path

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")

SRC = (Path(__file__).resolve().parent.parent / "fastddm_gb300" / "csrc" / "dft_consts.cuh").read_text()


def _array(name):
    m = re.search(name + r"\[\d+\] = \{([^}]*)\}", SRC)
    return [float(v.rstrip("f")) for v in m.group(1).split(",")]


def _scalar(name):
    return float(re.search(name + r" = ([^;]*);", SRC).group(1).rstrip("f"))


def test_odd_radix_tables():
    mpmath.mp.dps = 60
    ch, cl, sh, sl = (np.array(_array(n), dtype=np.float32) for n in ("kCosH", "kCosL", "kSinH", "kSinL"))
    cd, sd = np.array(_array("kCosD")), np.array(_array("kSinD"))
    idx = 0
    for R in (3, 5, 7, 11, 13):
        for k in range(R):
            c = mpmath.cos(2 * mpmath.pi * k / R)
            s = mpmath.sin(2 * mpmath.pi * k / R)
            assert cd[idx] == float(c) and sd[idx] == float(s)
            # hi is the nearest float, lo the nearest float to the remainder
            assert ch[idx] == np.float32(float(c)) and sh[idx] == np.float32(float(s))
            assert abs(float(c - (mpmath.mpf(float(ch[idx])) + mpmath.mpf(float(cl[idx]))))) <= 2.0 ** -48
            assert abs(float(s - (mpmath.mpf(float(sh[idx])) + mpmath.mpf(float(sl[idx]))))) <= 2.0 ** -48
            idx += 1
    assert idx == len(cd)


def test_sqrt_half():
    mpmath.mp.dps = 60
    r = mpmath.sqrt(mpmath.mpf(1) / 2)
    assert _scalar("kSqrtHalfD") == float(r)
    assert abs(float(r - mpmath.mpf(float(np.float32(_scalar("kSqrtHalfH")))) - mpmath.mpf(float(np.float32(_scalar("kSqrtHalfL")))))) <= 2.0 ** -48
