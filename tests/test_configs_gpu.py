"""Full-size parity of the benchmark configurations and of the reference's own fixture (needs a GPU).

* The reference test's fixture uncropped (``tests/test_ddm.py:14-16`` of the
  reference: 20 confocal frames of 256 x 256 uint8, lags 1..9) against the
  outputs of the reference's own Python core (``golden_confocal.npz``).
* 512 frames of 512 x 512 uint16 (2000 Brownian spots, D = 0.2 px^2/frame),
  Blackman-Harris window, all 511 lags: fft and diff mode in the float-float
  and FP64 tiers.
* 4000 frames of 64 x 64 uint8 with the 200 log-spaced lags of the
  4000-frame benchmark stack: the same temporal kernel configuration as
  4000 frames of 1024 x 1024 (transform length 8192, 200 lags).

Yardstick at these sizes: ``oracle.sampled_exact`` (direct FP64 DFTs of every
frame at sampled kx columns, D by direct differences), own error ~1e-12.
Tolerance: |got - exact| <= 1e-8 |exact| (ff) / 1e-9 (f64) elementwise on the
sampled modes, DC included; fft mode against diff mode on every mode within
1e-8 relative.  The benchmark metric's condition is 1e-6.
"""

import numpy as np
import pytest

import ddm_oracle as oracle
from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]

TOL = {"ff": 1e-8, "f64": 1e-9}


@pytest.fixture(scope="module")
def fddm(built_lib):
    import fastddm_gb300

    return fastddm_gb300


def _host(t):
    import torch

    return t.to(torch.int32).cpu().numpy()


def _sampled_check(data, imgs, lags, cols, window, precision, label):
    T, H, W = imgs.shape
    nx, ny = oracle.next_fast_len_cpp(W), oracle.next_fast_len_cpp(H)
    ex = oracle.sampled_exact(imgs, lags, nx, ny, cols, window)
    got = data[:, :, cols]
    err = np.abs(got - ex) / np.abs(ex)
    nodc = err.copy()
    nodc[:, ny // 2, list(cols).index(0)] = 0.0
    print(f"{label} {precision}: max rel err vs direct FP64 DFTs {err.max():.3e} (no DC {nodc.max():.3e}) "
          f"over {ny * len(cols)} modes")
    assert err.max() <= TOL[precision], (label, precision, float(err.max()))
    return float(err.max())


@pytest.mark.parametrize("precision", ["ff", "f64"])
@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_reference_fixture_full_size(fddm, golden_confocal, mode, precision):
    g = golden_confocal
    r = fddm.ddm(g["C_imgs"], g["C_lags"], mode=mode, precision=precision)
    ref = g[f"C_{mode}"]
    assert r._data.shape == ref.shape == (11, 256, 129)
    np.testing.assert_array_equal(r.kx, g["C_kx"])
    np.testing.assert_array_equal(r.ky, g["C_ky"])
    err = oracle.rel_err(r._data, ref)
    print(f"confocal 20 x 256^2 {mode} {precision}: max rel err vs reference {err:.3e}")
    assert err < 1e-10
    assert np.isclose(r._data, ref).all()  # the reference test's own criterion


def test_medium_stack_windowed_all_lags(fddm):
    """512 x 512^2 uint16, Blackman-Harris window, lags 1..511: fft and diff, ff and f64."""
    import torch

    from fastddm_gb300.synthetic import CONFIG2, make_stack_torch

    frames = make_stack_torch(CONFIG2, device="cuda")
    imgs = _host(frames).astype(np.uint16)
    T, H, W = imgs.shape
    lags = np.arange(1, T)
    w = fddm.window.blackman_harris(imgs.shape)
    cols = [0, 1, 3, 64, 128, 256]
    res = {}
    for precision in ("ff", "f64"):
        for mode in ("fft", "diff"):
            r = fddm.ddm(frames, lags, mode=mode, window=w, precision=precision)
            res[(mode, precision)] = r._data
            _sampled_check(r._data, imgs, lags, cols, w, precision, f"512x512^2 {mode}")
    for precision in ("ff", "f64"):
        a, b = res[("fft", precision)], res[("diff", precision)]
        e = oracle.rel_err(a, b)
        print(f"512x512^2 {precision}: fft vs diff over all {a.shape[1] * a.shape[2]} modes {e:.3e}")
        assert e <= TOL[precision]
    torch.cuda.empty_cache()


def test_long_stack_kernel_configuration(fddm):
    """4000 x 64^2 uint8 with the 200 log-spaced lags of the 4000-frame stack: transform length 8192."""
    from fastddm_gb300 import lags as flags
    from fastddm_gb300.synthetic import CONFIG3_TALL, make_stack_torch

    frames = make_stack_torch(CONFIG3_TALL, device="cuda")
    imgs = _host(frames).astype(np.uint8)
    T = imgs.shape[0]
    lags = np.unique(flags.logspace_int(T - 1, num=200, endpoint=True))
    cols = [0, 1, 2, 7, 16, 32]
    fft = fddm.ddm(frames, lags, mode="fft")._data
    diff = fddm.ddm(frames, lags, mode="diff")._data
    _sampled_check(fft, imgs, lags, cols, None, "ff", "4000x64^2 fft")
    _sampled_check(diff, imgs, lags, cols, None, "ff", "4000x64^2 diff")
    e = oracle.rel_err(fft, diff)
    print(f"4000x64^2: fft vs diff over all modes {e:.3e}")
    assert e <= TOL["ff"]


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_uint64_frames(fddm, mode):
    """64-bit unsigned input is converted to FP64 first, as the reference's cast does (ddm.cc:288-297)."""
    rng = np.random.default_rng(64)
    imgs = rng.integers(0, 1 << 40, size=(9, 12, 10), dtype=np.uint64)
    lags = [1, 2, 4, 8]
    r = fddm.ddm(imgs, lags, mode=mode)
    nx, ny = oracle.next_fast_len_cpp(10), oracle.next_fast_len_cpp(12)
    ex = oracle.ddm_exact(imgs.astype(np.float64), lags, nx, ny)
    assert oracle.rel_err(r._data, ex, floor=1e-10) < 1e-8


def test_not_enough_memory_is_refused(fddm, monkeypatch):
    """A job whose workspace and output exceed 90 % of free device memory is refused before any
    allocation, with the reference's message (memchk_gpu.cu:611-614)."""
    import torch

    from fastddm_gb300._ddm_b200 import DdmPlan

    torch.cuda.empty_cache()
    # a fake free-memory reading of 64 MiB; the job below needs ~8.5 GB
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda device=None: (64 << 20, 80 << 30))
    before = torch.cuda.memory_allocated()
    with pytest.raises(RuntimeError, match="Not enough memory"):
        DdmPlan("fft", 4000, 512, 512, 0, np.arange(1, 100), 512, 512, 8000, False, "ff", torch.device("cuda", 0))
    assert torch.cuda.memory_allocated() == before
    imgs = np.zeros((4000, 512, 512), dtype=np.uint8)
    with pytest.raises(RuntimeError, match="Not enough memory"):
        fddm.ddm(imgs, [1, 2, 3], mode="fft")
