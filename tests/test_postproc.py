"""Post-processing against the reference's own outputs (CPU).

``tests/golden/golden_post.npz`` holds the reference's ``estimate_camera_noise``
(every mode, on the image structure function of the reference fixture and on
its azimuthal average with and without errors) and ``azavg2isf_estimate``
results, written by ``tests/golden/make_golden_files.py``.  Everything except
the per-pixel "polyfit" mode (a GPU kernel, ``tests/test_postproc_gpu.py``) is
host numpy in the reference's operation order, so it must match bit for bit.
"""

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def post():
    return dict(np.load(GOLDEN / "golden_post.npz"))


@pytest.fixture(scope="module")
def objects(golden):
    from fastddm_gb300 import AzimuthalAverage, ImageStructureFunction, load

    tau = np.arange(1, 10, dtype=np.float64)
    sf = ImageStructureFunction(golden["A_fft"].copy(), golden["A_kx"], golden["A_ky"], 32, 48, tau, 0.65, 0.05)
    avg = load(str(GOLDEN / "golden_aa.aa.ddm"))
    plain = AzimuthalAverage(avg._data.copy(), None, avg.k.copy(), avg.tau.copy(), avg.bin_edges.copy())
    return sf, avg, plain


AA_CASES = {
    "zero": {}, "min": {}, "high_q": {}, "high_q_range": {"k_min": 2.0, "k_max": 0.5},
    "power_spec": {"k_min": 0.5, "k_max": 2.0}, "var": {"k_min": 0.5, "k_max": 2.0},
    "polyfit": {}, "polyfit7": {"num_points": 7},
}


@pytest.mark.parametrize("name", list(AA_CASES))
@pytest.mark.parametrize("tag", ["aa", "aa_noerr"])
def test_noise_azimuthal_average(objects, post, name, tag):
    from fastddm_gb300 import estimate_camera_noise

    _, avg, plain = objects
    obj = avg if tag == "aa" else plain
    mode = name.replace("_range", "").replace("7", "")
    if name == "high_q_range":
        with pytest.warns(UserWarning, match="swapped"):
            n, u = estimate_camera_noise(obj, mode=mode, **AA_CASES[name])
    else:
        n, u = estimate_camera_noise(obj, mode=mode, **AA_CASES[name])
    np.testing.assert_array_equal(n, post[f"{tag}_{name}_noise"])
    np.testing.assert_array_equal(u, post[f"{tag}_{name}_unc"])


@pytest.mark.parametrize("name", ["zero", "min", "min_mask", "high_q", "high_q_mask", "power_spec", "var"])
def test_noise_structure_function(objects, post, name):
    from fastddm_gb300 import estimate_camera_noise

    sf = objects[0]
    kw = {"zero": {}, "min": {}, "min_mask": {"mask": post["sf_mask"]}, "high_q": {},
          "high_q_mask": {"k_min": 0.5, "k_max": 2.5, "mask": post["sf_mask"]},
          "power_spec": {"k_min": 0.3, "k_max": 3.0}, "var": {"k_min": 0.3, "k_max": 3.0}}[name]
    n, u = estimate_camera_noise(sf, mode=name.replace("_mask", ""), **kw)
    np.testing.assert_array_equal(n, post[f"sf_{name}_noise"])
    np.testing.assert_array_equal(u, post[f"sf_{name}_unc"])


def test_noise_errors(objects):
    from fastddm_gb300 import estimate_camera_noise

    sf, avg, _ = objects
    with pytest.raises(RuntimeError, match="Unknown mode"):
        estimate_camera_noise(avg, mode="nope")
    with pytest.raises(TypeError):
        estimate_camera_noise(np.zeros(3), mode="zero")
    with pytest.warns(UserWarning, match="Casting to bool"):
        estimate_camera_noise(sf, mode="min", mask=np.ones(sf.shape[1:], dtype=np.int8))
    with pytest.raises(ValueError, match="exceed order"):
        estimate_camera_noise(sf, mode="polyfit", num_points=3)


@pytest.mark.parametrize("name", ["default", "min_ps", "custom"])
@pytest.mark.parametrize("tag", ["aa", "aa_noerr"])
def test_isf_estimate(objects, post, name, tag):
    from fastddm_gb300 import azavg2isf_estimate

    _, avg, plain = objects
    obj = avg if tag == "aa" else plain
    kw = {"default": {}, "min_ps": {"noise_est": "min", "plateau_est": "power_spec"},
          "custom": {"noise_est": "custom", "noise": post["isf_custom_noise"], "plateau_est": "custom",
                     "plateau": post["isf_custom_plateau"]}}[name]
    r = azavg2isf_estimate(obj, **kw)
    np.testing.assert_array_equal(r._data, post[f"isf_{name}_{tag}_data"])
    np.testing.assert_array_equal(r._err, post[f"isf_{name}_{tag}_err"])


def test_isf_estimate_errors_and_file(objects, tmp_path):
    from fastddm_gb300 import ISFReader, azavg2isf_estimate, load

    _, avg, _ = objects
    with pytest.raises(RuntimeError, match="Size of noise should be"):
        azavg2isf_estimate(avg, noise_est="custom", noise=np.ones(3))
    with pytest.raises(RuntimeError, match="Unsupported plateau_est"):
        azavg2isf_estimate(avg, plateau_est="nope")
    r = azavg2isf_estimate(avg)
    r.save(str(tmp_path / "isf"))
    assert (tmp_path / "isf.isf.ddm").read_bytes() == (GOLDEN / "golden_isf.isf.ddm").read_bytes()
    with ISFReader(str(GOLDEN / "golden_isf.isf.ddm")) as f:
        back = f.load()
    np.testing.assert_array_equal(back._data, r._data)
    np.testing.assert_array_equal(load(str(tmp_path / "isf.isf.ddm"))._err, r._err)
