"""Generate the binary file fixtures ``golden_sf.sf.ddm`` and ``golden_aa.aa.ddm``
with the reference's own writers.

The reference's ``SFWriter`` (``src/python/imagestructurefunction.py:409-627``)
and ``AAWriter`` (``src/python/azimuthalaverage.py:567-753``) are imported from
the reference source tree (as ``make_golden.py`` does) and write a small image
structure function (the reference fixture's structure function from
``golden.npz``, case A without window) and its azimuthal average.  The tests
check that this package writes the same bytes and reads these files back.

Usage (needs the reference checkout; the files it writes are committed):

    python tests/golden/make_golden_files.py /path/to/fastddm-reference
"""

from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import import_reference  # noqa: E402


def main(root: Path) -> None:
    import_reference(root)
    isf = importlib.import_module("fastddm.imagestructurefunction")
    aa = importlib.import_module("fastddm.azimuthalaverage")
    g = np.load(HERE / "golden.npz")
    data = np.ascontiguousarray(g["A_fft"])  # (L + 2, ny, nkx) = (11, 48, 17), frames 48 x 32
    L = data.shape[0] - 2
    tau = np.arange(1, L + 1, dtype=np.float64)
    sf = isf.ImageStructureFunction(data, g["A_kx"], g["A_ky"], 32, 48, tau, 0.65, 0.05)
    sf.save(str(HERE / "golden_sf"))
    # azimuthal average of the same object: the reference's own routine
    avg = aa.azimuthal_average(sf, bins=5, range=None, eval_err=True)
    avg.save(str(HERE / "golden_aa"))
    # the reference's eval_err=False path stops with an UnboundLocalError
    # (azimuthalaverage.py:438), so the error-free file is written from a
    # container built directly
    avg_noerr = aa.AzimuthalAverage(avg._data[:4].copy(), None, avg.k[:4].copy(), avg.tau.copy(), avg.bin_edges[:4].copy())
    avg_noerr.save(str(HERE / "golden_aa_noerr"))
    # post-processing on the same objects: the reference's estimate_camera_noise
    # (src/python/noise_est.py) and azavg2isf_estimate
    # (src/python/intermediatescatteringfunction.py:733-885)
    ne = importlib.import_module("fastddm.noise_est")
    isfm = importlib.import_module("fastddm.intermediatescatteringfunction")
    post = {}
    rng = np.random.default_rng(3)
    mask = rng.random(sf.shape[1:]) > 0.2
    kr = (0.5, 2.0)
    aa_cases = {
        "zero": {}, "min": {}, "high_q": {}, "high_q_range": {"k_min": kr[1], "k_max": kr[0]},
        "power_spec": {"k_min": kr[0], "k_max": kr[1]}, "var": {"k_min": kr[0], "k_max": kr[1]},
        "polyfit": {}, "polyfit7": {"num_points": 7},
    }
    avg_plain = aa.AzimuthalAverage(avg._data.copy(), None, avg.k.copy(), avg.tau.copy(), avg.bin_edges.copy())
    for tag, obj in (("aa", avg), ("aa_noerr", avg_plain)):
        for name, kw in aa_cases.items():
            mode = name.replace("_range", "").replace("7", "")
            n, u = ne.estimate_camera_noise(obj, mode=mode, **kw)
            post[f"{tag}_{name}_noise"], post[f"{tag}_{name}_unc"] = n, u
    sf_cases = {
        "zero": {}, "min": {}, "min_mask": {"mask": mask}, "high_q": {}, "high_q_mask": {"k_min": 0.5, "k_max": 2.5, "mask": mask},
        "power_spec": {"k_min": 0.3, "k_max": 3.0}, "var": {"k_min": 0.3, "k_max": 3.0},
        "polyfit": {}, "polyfit7": {"num_points": 7},
    }
    for name, kw in sf_cases.items():
        mode = name.replace("_mask", "").replace("7", "")
        n, u = ne.estimate_camera_noise(sf, mode=mode, **kw)
        post[f"sf_{name}_noise"], post[f"sf_{name}_unc"] = n, u
    post["sf_mask"] = mask
    isf_cases = {
        "default": {}, "min_ps": {"noise_est": "min", "plateau_est": "power_spec"},
        "custom": {"noise_est": "custom", "noise": np.linspace(1.0, 2.0, len(avg.k)), "plateau_est": "custom",
                   "plateau": 2 * avg.var + 3.0},
    }
    for name, kw in isf_cases.items():
        for tag, obj in (("aa", avg), ("aa_noerr", avg_plain)):
            r = isfm.azavg2isf_estimate(obj, **kw)
            post[f"isf_{name}_{tag}_data"] = r._data
            post[f"isf_{name}_{tag}_err"] = r._err
    post["isf_custom_noise"] = isf_cases["custom"]["noise"]
    post["isf_custom_plateau"] = isf_cases["custom"]["plateau"]
    isfm.azavg2isf_estimate(avg).save(str(HERE / "golden_isf"))
    np.savez_compressed(HERE / "golden_post.npz", **post)
    print("wrote", sorted(p.name for p in HERE.glob("golden_*")))


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
