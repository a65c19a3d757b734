"""Per-pixel "polyfit" camera-noise estimate on the device against the
reference's per-pixel numpy.polyfit results (needs a GPU).

The device kernel applies one least-squares operator to every pixel, where
numpy solves each pixel's system by SVD, so the results agree to rounding
(tolerance below), not bit for bit.
"""

from pathlib import Path

import numpy as np
import pytest

from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]
GOLDEN = Path(__file__).resolve().parent / "golden"
RTOL_NOISE, RTOL_UNC = 1e-9, 1e-6


@pytest.mark.parametrize("name,kw", [("polyfit", {}), ("polyfit7", {"num_points": 7})])
def test_polyfit_noise_matches_reference(built_lib, golden, name, kw):
    from fastddm_gb300 import ImageStructureFunction, estimate_camera_noise

    post = np.load(GOLDEN / "golden_post.npz")
    tau = np.arange(1, 10, dtype=np.float64)
    sf = ImageStructureFunction(golden["A_fft"].copy(), golden["A_kx"], golden["A_ky"], 32, 48, tau, 0.65, 0.05)
    n, u = estimate_camera_noise(sf, mode="polyfit", **kw)
    ref_n, ref_u = post[f"sf_{name}_noise"], post[f"sf_{name}_unc"]
    scale = np.max(np.abs(ref_n))
    np.testing.assert_allclose(n, ref_n, rtol=RTOL_NOISE, atol=1e-12 * scale)
    np.testing.assert_allclose(u, ref_u, rtol=RTOL_UNC, atol=1e-12 * scale)


def test_polyfit_noise_on_device_data(built_lib):
    """From the device copy ddm() keeps, against numpy.polyfit on sampled pixels; NaN rows stay NaN."""
    import fastddm_gb300 as fddm

    rng = np.random.default_rng(2)
    imgs = rng.poisson(150.0, size=(30, 40, 50)).astype(np.uint16)
    r = fddm.ddm(imgs, range(1, 20))
    n, u = fddm.estimate_camera_noise(r, mode="polyfit", num_points=6)
    x = r.tau[:6]
    for iy, ix in [(0, 0), (3, 7), (20, 25), (39, 25)]:
        p, pcov = np.polyfit(x, r.data[:6, iy, ix], deg=2, cov=True)
        assert np.isclose(n[iy, ix], p[-1], rtol=1e-9, atol=1e-12 * np.abs(r.data[:6]).max())
        assert np.isclose(u[iy, ix], np.sqrt(np.diag(pcov))[-1], rtol=1e-6)
    r._data[0, 5, 5] = np.nan
    r._device_data = None  # the host rows are uploaded instead
    n2, u2 = fddm.estimate_camera_noise(r, mode="polyfit", num_points=6)
    assert np.isnan(n2[5, 5]) and np.isnan(u2[5, 5])
    np.testing.assert_array_equal(np.delete(n2.ravel(), 5 * n.shape[1] + 5), np.delete(n.ravel(), 5 * n.shape[1] + 5))
