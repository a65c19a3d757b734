"""Generate the golden fixtures in ``tests/golden/golden.npz`` from the reference.

Runs the reference FastDDM's own Python code (the ``py`` core of
``src/python/_ddm_python.py``, ``azimuthalaverage.py``, ``window.py``,
``lags.py``, ``mask.py``, ``_fftopt.py``), imported from the reference source
tree, and stores its outputs together with the inputs.  The reference's
``tests/test_ddm.py`` checks that this core agrees with the ``cpp`` core
(``np.isclose``); the compiled cores themselves are not built here.

It writes ``golden.npz`` (small cases and helper tables) and
``golden_confocal.npz`` (the reference test's 20 confocal frames of 256 x 256
at full size, lags 1..9, fft and diff mode).

Usage (needs the reference checkout; the fixtures it writes are committed):

    python tests/golden/make_golden.py /path/to/fastddm-reference
"""

from __future__ import annotations

import importlib
import struct
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def import_reference(root: Path):
    """Import the reference's pure-Python modules without its compiled extensions."""
    src = root / "src" / "python"
    pkg = types.ModuleType("fastddm")
    pkg.__path__ = [str(src)]
    sys.modules["fastddm"] = pkg
    cfg = types.ModuleType("fastddm._config")
    cfg.IS_CPP_ENABLED = False
    cfg.IS_CUDA_ENABLED = False
    cfg.IS_SINGLE_PRECISION = False
    cfg.CUDA_VERSION = ""
    cfg.DTYPE = np.float64
    sys.modules["fastddm._config"] = cfg
    # image-file readers are not on the path and their dependencies are absent
    for name in ["tifffile", "skimage", "skimage.io", "nd2reader"]:
        sys.modules[name] = types.ModuleType(name)
    sys.modules["nd2reader"].ND2Reader = object
    mods = {}
    for name in ["_ddm", "azimuthalaverage", "window", "lags", "mask", "_fftopt"]:
        mods[name] = importlib.import_module(f"fastddm.{name}")
    return mods


def read_tiff_u8(path: Path) -> np.ndarray:
    """Uncompressed single-strip 8-bit grayscale TIFF (the confocal test images)."""
    d = path.read_bytes()
    bo = ">" if d[:2] == b"MM" else "<"
    off = struct.unpack(bo + "I", d[4:8])[0]
    n = struct.unpack(bo + "H", d[off:off + 2])[0]
    tags = {}
    for i in range(n):
        e = d[off + 2 + 12 * i: off + 14 + 12 * i]
        tag, typ, cnt = struct.unpack(bo + "HHI", e[:8])
        val = struct.unpack(bo + "H", e[8:10])[0] if typ == 3 else struct.unpack(bo + "I", e[8:12])[0]
        tags[tag] = val
    w, h, bits, comp, strip = tags[256], tags[257], tags[258], tags[259], tags[273]
    assert bits == 8 and comp == 1
    return np.frombuffer(d[strip:strip + w * h], dtype=np.uint8).reshape(h, w)


def main(root: Path) -> None:
    ref = import_reference(root)
    ddm = ref["_ddm"].ddm
    aa = ref["azimuthalaverage"]
    g = {}

    # case A: the reference test fixture (confocal frames 0..19, lags 1..9),
    # cropped to 48 x 32 to keep the fixture small
    files = sorted((root / "tests" / "test-imgs" / "confocal").glob("*.tif"))[:20]
    imgs = np.stack([read_tiff_u8(p) for p in files])[:, 100:148, 60:92].copy()
    lags = np.arange(1, 10)
    g["A_imgs"] = imgs
    g["A_lags"] = lags
    win = ref["window"].blackman_harris(imgs.shape)
    g["A_window"] = win
    for mode in ("fft", "diff"):
        r = ddm(imgs, lags, core="py", mode=mode)
        g[f"A_{mode}"] = r._data
        g[f"A_{mode}_win"] = ddm(imgs, lags, core="py", mode=mode, window=win)._data
    g["A_kx"], g["A_ky"] = r.kx, r.ky
    base = ddm(imgs, lags, core="py", mode="fft")
    bins = len(base.ky) // 2
    ccm = ref["mask"].central_cross_mask(base.shape[1:])
    a1 = aa.azimuthal_average(base, bins=bins, range=(0, base.ky[-1]), mask=ccm)
    edges = np.linspace(0, base.ky[-1], num=bins).tolist()
    a2 = aa.azimuthal_average(base, bins=edges, mask=ccm)
    for tag, a in (("A_aa", a1), ("A_aa_edges", a2)):
        g[f"{tag}_data"], g[f"{tag}_err"], g[f"{tag}_k"], g[f"{tag}_edges"] = a._data, a._err, a.k, a.bin_edges
    # weighted average without a mask, default bins and range
    wts = np.linspace(0.0, 2.0, base.shape[1] * base.shape[2]).reshape(base.shape[1:])
    a3 = aa.azimuthal_average(base, bins=7, weights=wts)
    g["A_aa_w_data"], g["A_aa_w_err"], g["A_aa_w_k"], g["A_aa_w_edges"] = a3._data, a3._err, a3.k, a3.bin_edges
    g["A_aa_w_weights"] = wts

    # case B: seeded odd/padded sizes, 16-bit, Blackman window, sparse lags
    rng = np.random.default_rng(1234)
    T, H, W = 12, 21, 17
    yy, xx = np.mgrid[0:H, 0:W]
    frames = []
    for t in range(T):
        cx, cy = 6 + 0.4 * t, 9 - 0.3 * t
        scene = 300 + 2500 * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / 8.0)
        frames.append(rng.poisson(scene))
    imgsB = np.clip(np.stack(frames), 0, 65535).astype(np.uint16)
    lagsB = np.array([1, 2, 3, 5, 8, 11])
    winB = ref["window"].blackman(imgsB.shape)
    g["B_imgs"], g["B_lags"], g["B_window"] = imgsB, lagsB, winB
    for mode in ("fft", "diff"):
        r = ddm(imgsB, lagsB, core="py", mode=mode, window=winB)
        g[f"B_{mode}"] = r._data
    g["B_kx"], g["B_ky"] = r.kx, r.ky
    g["B_nx"], g["B_ny"] = r.width, r.height

    # tables of the small helpers
    fo = ref["_fftopt"]
    targets = np.arange(1, 3001)
    g["nfl_cpp"] = np.array([fo.next_fast_len(int(t), "cpp") for t in targets])
    g["nfl_cuda"] = np.array([fo.next_fast_len(int(t), "cuda") for t in targets])
    g["nfl_cuda_even"] = np.array([fo.next_fast_len(int(t), "cuda", True) for t in targets])
    lg = ref["lags"]
    for stop, num, ep in ((10, 5, True), (10, 5, False), (3999, 200, True), (511, 50, False), (1000, 100, True)):
        g[f"logspace_{stop}_{num}_{int(ep)}"] = lg.logspace_int(stop, num=num, endpoint=ep)
    g["fib_13_1"] = lg.fibonacci(13, endpoint=True)
    g["fib_100_0"] = lg.fibonacci(100)
    for shape in ((5, 7), (16, 16), (3, 24, 9)):
        key = "x".join(map(str, shape))
        g[f"win_blackman_{key}"] = ref["window"].blackman(shape)
        g[f"win_bh_{key}"] = ref["window"].blackman_harris(shape)
    g["ccm_48x17"] = ref["mask"].central_cross_mask((48, 17))
    kx = 2 * np.pi * np.fft.fftfreq(16)[:9]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(12))
    g["ccm_k_12x9"] = ref["mask"].central_cross_mask((12, 9), kx, ky)

    np.savez_compressed(HERE / "golden.npz", **g)
    print("wrote", HERE / "golden.npz", sum(np.asarray(v).nbytes for v in g.values()), "bytes raw")

    # case C: the reference test fixture at its full size, uncropped: confocal
    # frames 0..19 of 256 x 256, lags 1..9 (tests/test_ddm.py:14-16), both modes
    full = np.stack([read_tiff_u8(p) for p in files])
    c = {"C_imgs": full, "C_lags": lags}
    for mode in ("fft", "diff"):
        r = ddm(full, lags, core="py", mode=mode)
        c[f"C_{mode}"] = r._data
    c["C_kx"], c["C_ky"] = r.kx, r.ky
    np.savez_compressed(HERE / "golden_confocal.npz", **c)
    print("wrote", HERE / "golden_confocal.npz", sum(np.asarray(v).nbytes for v in c.values()), "bytes raw")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference"))
