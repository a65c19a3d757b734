"""The GB300 azimuthal average against the reference's loops (needs a GPU).

The device kernel sums every (bin, row) in the reference's pixel order with the
reference's operation order in IEEE FP64, so the comparison is bit-exact.
"""

import numpy as np
import pytest

import ddm_oracle as oracle
from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def fddm(built_lib):
    import fastddm_gb300

    return fastddm_gb300


def _isf(fddm, golden):
    from fastddm_gb300.imagestructurefunction import ImageStructureFunction

    return ImageStructureFunction(golden["A_fft"].copy(), golden["A_kx"].copy(), golden["A_ky"].copy(), 32, 48,
                                  np.arange(1.0, 10.0))


def _same(a, b):
    np.testing.assert_array_equal(a, b)


def test_reference_fixture_bins(fddm, golden):
    """tests/test_ddm.py:26-31 of the reference: bins = ny // 2 over (0, ky[-1]), central cross masked."""
    isf = _isf(fddm, golden)
    ccm = fddm.mask.central_cross_mask(isf.shape[1:])
    a = fddm.azimuthal_average(isf, bins=len(isf.ky) // 2, range=(0, isf.ky[-1]), mask=ccm)
    _same(a._data, golden["A_aa_data"])
    _same(a._err, golden["A_aa_err"])
    _same(a.k, golden["A_aa_k"])
    _same(a.bin_edges, golden["A_aa_edges"])


def test_bin_edge_list_equals_int_bins(fddm, golden):
    """tests/test_ddm.py:175-182 of the reference."""
    isf = _isf(fddm, golden)
    ccm = fddm.mask.central_cross_mask(isf.shape[1:])
    bins = len(isf.ky) // 2
    a = fddm.azimuthal_average(isf, bins=bins, range=(0, isf.ky[-1]), mask=ccm)
    b = fddm.azimuthal_average(isf, bins=np.linspace(0, isf.ky[-1], num=bins).tolist(), mask=ccm)
    assert np.isclose(a._data, b._data, equal_nan=True).all()
    _same(b._data, golden["A_aa_edges_data"])
    _same(b._err, golden["A_aa_edges_err"])


def test_weights_default_range(fddm, golden):
    isf = _isf(fddm, golden)
    a = fddm.azimuthal_average(isf, bins=7, weights=golden["A_aa_w_weights"])
    _same(a._data, golden["A_aa_w_data"])
    _same(a._err, golden["A_aa_w_err"])
    _same(a.k, golden["A_aa_w_k"])


@pytest.mark.parametrize("shape,bins", [((5, 24, 13), 9), ((3, 31, 16), 40), ((4, 16, 9), 3)])
def test_random_maps_vs_loops(fddm, shape, bins):
    """Odd/even widths, empty bins (NaN), zero-weight pixels, single-pixel bins."""
    rng = np.random.default_rng(shape[1])
    data = rng.random(shape) * 10.0
    ny, nkx = shape[1:]
    width = 2 * (nkx - 1) + (shape[1] % 2)
    kx = 2 * np.pi * np.fft.fftfreq(width)[: width // 2 + 1]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(ny))
    from fastddm_gb300.imagestructurefunction import ImageStructureFunction

    isf = ImageStructureFunction(data, kx, ky, width, ny, np.arange(1.0, shape[0] - 1.0))
    w = rng.random((ny, nkx))
    w[w < 0.2] = 0.0
    mask = rng.random((ny, nkx)) > 0.1
    a = fddm.azimuthal_average(isf, bins=bins, mask=mask, weights=w)
    ref = oracle.azimuthal_average(data, kx, ky, width, bins, None, mask, w)
    _same(a._data, ref[0])
    _same(a._err, ref[1])
    _same(a.k, ref[2])
    _same(a.bin_edges, ref[3])


def test_without_error(fddm, golden):
    isf = _isf(fddm, golden)
    a = fddm.azimuthal_average(isf, bins=12, eval_err=False)
    assert a._err is None and a.err is None
    ref = oracle.azimuthal_average(isf._data, isf.kx, isf.ky, isf.width, 12, eval_err=False)
    _same(a._data, ref[0])


def test_on_device_result(fddm, golden):
    """The structure function produced by core='b200' keeps its device copy; the average uses it."""
    imgs, lags = golden["A_imgs"], golden["A_lags"]
    r = fddm.ddm(imgs, lags)
    assert r._device_data is not None
    a = fddm.azimuthal_average(r, bins=10)
    ref = oracle.azimuthal_average(r._data, r.kx, r.ky, r.width, 10)
    _same(a._data, ref[0])
    _same(a._err, ref[1])


@pytest.mark.parametrize("shape,bins", [((5, 24, 13), 9), ((3, 31, 16), 40), ((6, 96, 49), 64)])
def test_fast_order_within_rounding_of_the_loops(fddm, shape, bins):
    """exact=False (a warp of fused multiply-adds per bin and row) against the reference's loops: the same
    empty bins (NaN), relative differences within 1e-12, and the same result on every run."""
    rng = np.random.default_rng(shape[1] + 7)
    data = rng.random(shape) * 10.0 + 1.0
    ny, nkx = shape[1:]
    width = 2 * (nkx - 1) + (shape[1] % 2)
    kx = 2 * np.pi * np.fft.fftfreq(width)[: width // 2 + 1]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(ny))
    from fastddm_gb300.imagestructurefunction import ImageStructureFunction

    isf = ImageStructureFunction(data, kx, ky, width, ny, np.arange(1.0, shape[0] - 1.0))
    w = rng.random((ny, nkx)) + 0.5
    mask = rng.random((ny, nkx)) > 0.1
    fast = fddm.azimuthal_average(isf, bins=bins, mask=mask, weights=w, exact=False)
    again = fddm.azimuthal_average(isf, bins=bins, mask=mask, weights=w, exact=False)
    ref = oracle.azimuthal_average(data, kx, ky, width, bins, None, mask, w)
    _same(fast._data, again._data)
    _same(fast._err, again._err)
    for got, want in ((fast._data, ref[0]), (fast._err, ref[1])):
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        np.testing.assert_allclose(got[ok], want[ok], rtol=1e-12, atol=0.0)
    _same(fast.k, ref[2])
