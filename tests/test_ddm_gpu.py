"""Parity of the GB300 structure-function kernels with the FP64 oracle (needs a GPU).

Yardstick: ``oracle.ddm_exact`` (extended precision, no cancellation).  The
FP64 restatements of the reference's ``cpp`` algorithms are themselves off by
up to ~1e-7 (fft mode, S1 + S2 - 2 Re C at the DC mode) and ~1e-8 (VAR =
PS - |<F>|^2) on these inputs, so they are checked with the reference's own
cross-core criterion, np.isclose (rtol 1e-5, atol 1e-8).

Tolerances, elementwise over every output row (DC included):
    |got - exact| <= RTOL * |exact| + ATOL * max|exact row|
  ff  (float-float FFTs and sums)   RTOL 1e-8, ATOL 1e-13
  f64 (native FP64)                 RTOL 1e-9, ATOL 1e-15
  f32 (FP32 FFTs, float-float sums) RTOL 5e-2, ATOL 1e-6  (FP32 FFTs cannot reach 1e-6)
ATOL only matters where the exact value is 0 (e.g. Nyquist modes of tiny frames).
"""

import numpy as np
import pytest

import ddm_oracle as oracle
from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]

TOL = {"ff": 1e-8, "f64": 1e-9, "f32": 5e-2}
ATOL = {"ff": 1e-13, "f64": 1e-15, "f32": 1e-6}


@pytest.fixture(scope="module")
def fddm(built_lib):
    import fastddm_gb300

    return fastddm_gb300


def _oracle(imgs, lags, mode, window=None):
    """FP64 restatement of the reference's cpp algorithm for `mode`."""
    T, H, W = imgs.shape
    nx, ny = oracle.next_fast_len_cpp(W), oracle.next_fast_len_cpp(H)
    lags = oracle.prepare_lags(lags, T)
    if mode == "fft":
        return oracle.ddm_fft(imgs, lags, nx, ny, oracle.next_fast_len_cpp(2 * T), window)
    return oracle.ddm_diff(imgs, lags, nx, ny, window)


def _exact(imgs, lags, window=None):
    T, H, W = imgs.shape
    nx, ny = oracle.next_fast_len_cpp(W), oracle.next_fast_len_cpp(H)
    return oracle.ddm_exact(imgs, oracle.prepare_lags(lags, T), nx, ny, window)


def _check(data, imgs, lags, mode, precision, window=None, label=""):
    ex = _exact(imgs, lags, window)
    rowmax = np.abs(ex).reshape(ex.shape[0], -1).max(axis=1)[:, None, None]
    dev = np.abs(data - ex)
    ok = dev <= TOL[precision] * np.abs(ex) + ATOL[precision] * rowmax
    err = oracle.rel_err(data, ex, floor=1e-10)
    print(f"{label} {mode} {precision}: max rel err vs exact {err:.3e}, max abs/rowmax {np.max(dev / np.maximum(rowmax, 1e-300)):.3e}")
    assert ok.all(), (label, mode, precision, err)
    if precision != "f32":
        assert np.isclose(data, _oracle(imgs, lags, mode, window)).all()


def _poisson_stack(shape, dtype, seed=0, level=300.0):
    rng = np.random.default_rng(seed)
    T, H, W = shape
    yy, xx = np.mgrid[0:H, 0:W]
    frames = []
    for t in range(T):
        cx, cy = (0.3 + 0.01 * t) * W, (0.6 - 0.01 * t) * H
        scene = level + 8 * level * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (0.02 * H * W + 2))
        frames.append(rng.poisson(scene))
    a = np.stack(frames)
    if np.dtype(dtype).kind in "ui":
        info = np.iinfo(dtype)
        a = np.clip(a, info.min, info.max)
    return a.astype(dtype)


@pytest.mark.parametrize("precision", ["ff", "f64", "f32"])
@pytest.mark.parametrize("mode", ["fft", "diff"])
@pytest.mark.parametrize("case,winkey,outkey", [
    ("A", None, "A_{mode}"),
    ("A", "A_window", "A_{mode}_win"),
    ("B", "B_window", "B_{mode}"),
])
def test_golden_vectors(fddm, golden, precision, mode, case, winkey, outkey):
    """The reference's own test fixture (confocal frames, lags 1..9) and a padded odd-size case."""
    imgs, lags = golden[f"{case}_imgs"], golden[f"{case}_lags"]
    w = golden[winkey] if winkey else None
    r = fddm.ddm(imgs, lags, mode=mode, window=w, precision=precision)
    ref = golden[outkey.format(mode=mode)]
    assert r._data.shape == ref.shape
    np.testing.assert_array_equal(r.kx, golden[f"{case}_kx"])
    np.testing.assert_array_equal(r.ky, golden[f"{case}_ky"])
    err = oracle.rel_err(r._data, ref)
    print(f"{case} {mode} {precision} window={winkey is not None}: max rel err vs reference {err:.3e}")
    assert err < max(TOL[precision], 2e-11)
    if precision != "f32":
        assert np.isclose(r._data, ref).all()
    _check(r._data, imgs, lags, mode, precision, w, label=f"golden {case}")


@pytest.mark.parametrize("precision", ["ff", "f64"])
@pytest.mark.parametrize("mode", ["fft", "diff"])
@pytest.mark.parametrize("dtype", ["uint8", "int16", "uint16", "int32", "uint32", "float32", "float64", "int64"])
def test_dtypes(fddm, precision, mode, dtype):
    imgs = _poisson_stack((10, 16, 24), dtype, seed=3, level=20.0 if dtype == "uint8" else 300.0)
    lags = [1, 2, 4, 9]
    r = fddm.ddm(imgs, lags, mode=mode, precision=precision)
    _check(r._data, imgs, lags, mode, precision, label=dtype)


@pytest.mark.parametrize("shape", [(12, 33, 64), (10, 32, 32), (6, 7, 16)])
def test_uint8_staged_rows(fddm, shape):
    """8-bit frames with power-of-two widths, staged rows and no window take the row pass's
    four-pixels-per-load path (odd heights leave the last pair half empty)."""
    imgs = _poisson_stack(shape, "uint8", seed=sum(shape), level=30.0)
    lags = sorted({1, 2, shape[0] // 2, shape[0] - 1})
    for mode in ("fft", "diff"):
        r = fddm.ddm(imgs, lags, mode=mode)
        _check(r._data, imgs, lags, mode, "ff", label=f"u8 {shape}")


@pytest.mark.parametrize("shape", [
    (7, 13, 11),     # radices 13 and 11, nt = 14 (2 x 7)
    (9, 25, 49),     # 5 x 5 and 7 x 7
    (33, 30, 45),    # odd width -> nx = 45, nt = 66
    (16, 19, 23),    # padded: 19 -> 20, 23 -> 24
    (40, 64, 96),    # 96 = 2^5 x 3
    (3, 2, 2),       # tiny frames
])
@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_shapes_and_radices(fddm, shape, mode):
    imgs = _poisson_stack(shape, "uint16", seed=sum(shape))
    T = shape[0]
    lags = sorted({1, 2, T // 2, T - 1})
    w = fddm.window.blackman_harris(shape)
    for window in (None, w):
        r = fddm.ddm(imgs, lags, mode=mode, window=window, precision="ff")
        _check(r._data, imgs, lags, mode, "ff", window, label=f"{shape} window={window is not None}")


@pytest.mark.parametrize("T", [3, 10, 500, 1000, 2000, 6000])
def test_long_sequences_and_first_radix(fddm, T):
    """Temporal transforms whose plans start with radix 2, 4 and 8 (N = 6, 20,
    1024, 2048, 4096, 12288), up to 6000 frames on one CTA per mode."""
    imgs = _poisson_stack((T, 4, 6), "uint16", seed=T)
    lags = np.unique(np.concatenate([np.geomspace(1, T - 1, 40).astype(int), [T - 40, T - 33, T - 32, T - 1]]))
    lags = lags[(lags >= 1) & (lags < T)]
    r = fddm.ddm(imgs, lags, mode="fft", precision="ff")
    _check(r._data, imgs, lags, "fft", "ff", label=f"T={T}")


def _long_lags(T, n=30):
    lags = np.unique(np.concatenate([np.geomspace(1, T - 1, n).astype(int), [T - 40, T - 33, T - 32, T - 1]]))
    return lags[(lags >= 1) & (lags < T)]


@pytest.mark.parametrize("split", [2, 4, 8])
@pytest.mark.parametrize("T", [3, 40, 333, 1000])
def test_split_temporal_kernel(fddm, monkeypatch, T, split):
    """The long-series fft kernel (first pass in global memory, sub-transforms
    of N/split in shared memory), forced on short series for every first radix."""
    monkeypatch.setenv("FDDM_B200_TEMPORAL_SPLIT", str(split))
    imgs = _poisson_stack((T, 5, 6), "uint16", seed=T + split)
    lags = _long_lags(T)
    w = fddm.window.blackman_harris((5, 6))
    for precision in ("ff", "f64"):
        r = fddm.ddm(imgs, lags, mode="fft", window=w, precision=precision)
        _check(r._data, imgs, lags, "fft", precision, w, label=f"split {split} T={T}")


@pytest.mark.parametrize("T", [1, 2, 3, 4, 5, 6, 8, 9])
def test_tiny_sequences_fft(fddm, T):
    """Very short series: single-pass temporal plans (T = 1, 2, 4), whose padded first
    pass reads an all-ones twiddle table, and lags all in the direct tail."""
    imgs = _poisson_stack((T, 6, 8), "uint16", seed=T)
    lags = list(range(1, T))
    for precision in ("ff", "f64"):
        if T == 1:
            with pytest.warns(UserWarning):
                r = fddm.ddm(imgs, [0], mode="fft", precision=precision)
        else:
            r = fddm.ddm(imgs, lags, mode="fft", precision=precision)
        _check(r._data, imgs, lags, "fft", precision, label=f"tiny T={T}")


def test_lag_order_at_the_c_abi(fddm):
    """fft mode needs strictly increasing lags (the transform path pairs them with
    prefix sums by position and sums the last ones directly from the end of the
    list); diff mode returns rows in the given order."""
    from fastddm_gb300 import _ddm_b200
    from fastddm_gb300._lib import FddmError

    imgs = _poisson_stack((12, 8, 10), "uint16", seed=4)
    with pytest.raises(FddmError, match="strictly increasing"):
        _ddm_b200.ddm_device(imgs, [5, 1, 3], 10, 8, 32, mode="fft")
    with pytest.raises(FddmError, match="strictly increasing"):
        _ddm_b200.ddm_device(imgs, [1, 3, 3], 10, 8, 32, mode="fft")
    got = _ddm_b200.ddm_device(imgs, [5, 1, 3], 10, 8, 0, mode="diff").cpu().numpy()
    ex = _exact(imgs, [1, 3, 5])
    np.testing.assert_allclose(got[[1, 2, 0]], ex[:3], rtol=1e-8, atol=1e-13 * np.abs(ex).max())


@pytest.mark.parametrize("T,mode,precision", [
    (7000, "fft", "ff"),     # just past the single-CTA transform: split kernel
    (20000, "fft", "ff"),
    (20000, "fft", "f32"),   # f32 switches to the split kernel later (8-byte values)
    (20000, "diff", "ff"),   # series read from global memory
])
def test_long_sequences(fddm, T, mode, precision):
    imgs = _poisson_stack((T, 4, 6), "uint8", seed=T, level=40.0)
    lags = _long_lags(T, 20)
    r = fddm.ddm(imgs, lags, mode=mode, precision=precision)
    _check(r._data, imgs, lags, mode, precision, label=f"T={T}")


def test_long_sequence_window_odd_size_f64(fddm):
    """Split temporal transform with a window, odd frame sizes (padded FFTs) and the f64 tier."""
    T = 7001
    imgs = _poisson_stack((T, 5, 7), "uint16", seed=5)
    lags = _long_lags(T, 15)
    w = fddm.window.blackman((5, 7))
    for precision in ("ff", "f64"):
        r = fddm.ddm(imgs, lags, mode="fft", window=w, precision=precision)
        _check(r._data, imgs, lags, "fft", precision, w, label=f"T={T} window")


def test_sequence_beyond_the_split_kernel_is_refused(fddm):
    from fastddm_gb300._lib import FddmError

    imgs = np.zeros((40000, 2, 2), dtype=np.uint8)
    with pytest.raises(FddmError, match="too long"):
        fddm.ddm(imgs, [1, 2], mode="fft")


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_chunked_host_result_equals_device_result(fddm, mode):
    """With a host result the temporal stage runs in chunks of modes whose columns are copied to
    the host while the next chunk computes; the host array must equal the device array."""
    imgs = _poisson_stack((24, 96, 128), "uint16", seed=3)  # 6240 modes: chunked
    r = fddm.ddm(imgs, [1, 2, 5, 11, 23], mode=mode)
    np.testing.assert_array_equal(r._data, r._device_data.cpu().numpy())
    _check(r._data, imgs, [1, 2, 5, 11, 23], mode, "ff", label="chunked")


def test_concurrent_calls(fddm):
    """Calls from several threads at once give the same results as sequential calls."""
    from concurrent.futures import ThreadPoolExecutor

    stacks = [_poisson_stack((32, 48, 64), "uint16", seed=s) for s in range(4)]
    lags = [1, 2, 7, 31]
    ref = [fddm.ddm(x, lags)._data for x in stacks]
    with ThreadPoolExecutor(max_workers=4) as ex:
        got = list(ex.map(lambda x: fddm.ddm(x, lags)._data, stacks * 2))
    for i, g in enumerate(got):
        np.testing.assert_array_equal(g, ref[i % 4])


def test_config1_all_lags_fft_vs_oracle_and_diff(fddm):
    """64 frames of 128 x 128 uint16 Brownian spots, lags 1..63, no window."""
    from fastddm_gb300.synthetic import CONFIG1, make_stack

    imgs = make_stack(CONFIG1)
    lags = np.arange(1, 64)
    fft = fddm.ddm(imgs, lags, mode="fft")._data
    diff = fddm.ddm(imgs, lags, mode="diff")._data
    exact = _exact(imgs, lags)
    ref_fft = _oracle(imgs, lags, "fft")
    ref_diff = _oracle(imgs, lags, "diff")
    e = {
        "fft_vs_exact": oracle.rel_err(fft, exact),
        "diff_vs_exact": oracle.rel_err(diff, exact),
        "fft_vs_diff": oracle.rel_err(fft, diff),
        "fft_vs_cpp_fft": oracle.rel_err(fft, ref_fft),
        "fft_vs_cpp_fft_noDC": oracle.rel_err(fft, ref_fft, skip_dc=True),
        "fft_vs_cpp_diff": oracle.rel_err(fft, ref_diff),
        "cpp_fft_vs_exact": oracle.rel_err(ref_fft, exact),
    }
    print(e)
    # the 1e-6 target against FP64, met against every reference
    assert all(v < 1e-6 for v in e.values()), e
    assert e["fft_vs_exact"] < TOL["ff"] and e["diff_vs_exact"] < TOL["ff"]


def test_edge_cases(fddm):
    imgs = _poisson_stack((6, 8, 10), "uint16")
    # only lag 0 -> removed, output holds PS and VAR only
    with pytest.warns(UserWarning):
        r = fddm.ddm(imgs, [0], mode="fft")
    assert r._data.shape == (2, 8, 6)
    _check(r._data, imgs, [], "fft", "ff", label="no lags")
    # a single frame: no lags at all
    one = imgs[:1]
    with pytest.warns(UserWarning):
        r1 = fddm.ddm(one, [0], mode="diff")
    np.testing.assert_allclose(r1.var, 0.0, atol=1e-9 * np.max(r1.power_spec))
    # duplicated / unsorted lags are deduplicated and sorted
    r2 = fddm.ddm(imgs, [5, 1, 3, 1], mode="fft")
    np.testing.assert_array_equal(r2.tau, [1.0, 3.0, 5.0])
    _check(r2._data, imgs, [1, 3, 5], "fft", "ff", label="dedup")


def test_repeat_calls_identical(fddm):
    """Same input, same plan: bitwise identical results (no atomics in the pipeline)."""
    imgs = _poisson_stack((20, 32, 32), "uint16", seed=7)
    a = fddm.ddm(imgs, range(1, 20), mode="fft")._data
    b = fddm.ddm(imgs, range(1, 20), mode="fft")._data
    np.testing.assert_array_equal(a, b)


def test_backend_function_contract(fddm):
    """The registry functions take the reference's positional arguments and return the raw array."""
    imgs = _poisson_stack((8, 12, 16), "uint8", level=30.0)
    lags = np.array([1, 3])
    out = fddm._backend["b200"]["fft"](imgs, lags, 16, 12, 16, np.array([], dtype=np.float64))
    assert out.dtype == np.float64 and out.shape == (4, 12, 9)
    out2 = fddm._backend["b200"]["diff"](imgs, lags, 16, 12, np.array([], dtype=np.float64), gpu_id=0)
    assert oracle.rel_err(out, out2) < 1e-9


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_page_locked_frames_read_in_place_or_uploaded(fddm, built_lib, monkeypatch, mode):
    """Page-locked host frames are read by the row pass in place (no copy-engine upload, no device
    copy of the stack); FDDM_B200_ZERO_COPY=0 uploads them chunk by chunk instead: identical results.
    Rows that are not a multiple of 16 bytes cannot be read in place and are uploaded."""
    import torch

    imgs = _poisson_stack((40, 72, 64), "uint8", seed=21, level=30.0)
    lags = [1, 2, 5, 13, 39]
    pinned = torch.from_numpy(imgs).pin_memory()
    direct = fddm.ddm(pinned, lags, mode=mode)._data
    assert built_lib.fddm_b200_last_input_path() == 1
    monkeypatch.setenv("FDDM_B200_ZERO_COPY", "0")
    uploaded = fddm.ddm(pinned, lags, mode=mode)._data
    assert built_lib.fddm_b200_last_input_path() == 2
    monkeypatch.delenv("FDDM_B200_ZERO_COPY")
    np.testing.assert_array_equal(direct, uploaded)
    _check(direct, imgs, lags, mode, "ff", label="page-locked in place")
    # 60-byte rows: the in-place read is refused before any work, the frames are uploaded
    odd = torch.from_numpy(np.ascontiguousarray(imgs[:, :, :60])).pin_memory()
    r = fddm.ddm(odd, lags, mode=mode)._data
    assert built_lib.fddm_b200_last_input_path() == 2
    np.testing.assert_array_equal(r, fddm.ddm(np.ascontiguousarray(imgs[:, :, :60]), lags, mode=mode)._data)
    fddm.ddm(imgs, lags, mode=mode)
    assert built_lib.fddm_b200_last_input_path() == 2  # pageable numpy: uploaded
    fddm.ddm(pinned.cuda(), lags, mode=mode)
    assert built_lib.fddm_b200_last_input_path() == 0  # device frames


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_input_paths_agree(fddm, mode):
    """Pageable numpy, page-locked CPU tensor (overlapped upload) and CUDA tensor inputs give identical results."""
    import torch

    imgs = _poisson_stack((48, 40, 56), "uint16", seed=11)
    lags = [1, 2, 3, 7, 20, 47]
    a = fddm.ddm(imgs, lags, mode=mode)._data
    pinned = torch.from_numpy(imgs.astype(np.int32)).to(torch.int16).pin_memory()
    b = fddm.ddm(pinned, lags, mode=mode)._data
    c = fddm.ddm(pinned.cuda(), lags, mode=mode)._data
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    _check(a, imgs, lags, mode, "ff", label="input paths")


@pytest.mark.parametrize("precision", ["ff", "f64", "f32"])
@pytest.mark.parametrize("T", [4000, 2000, 700, 64, 3])
def test_fused_radix2_temporal_path_is_bitwise_identical(fddm, monkeypatch, T, precision):
    """Plans with first radix 2 fold the padded first pass into the pass over the series and run the
    last forward pass, the pairing and the first inverse pass as one step: the same operations in
    the same order.  Float-float arithmetic is written with explicitly rounded operations, so its
    results equal those of the separate passes bit for bit; the native FP64 and FP32 tiers leave
    multiply-add contraction to the compiler, which may differ between the two code paths."""
    imgs = _poisson_stack((T, 6, 8), "uint16", seed=T)
    lags = _long_lags(T, 25) if T > 40 else list(range(1, T))
    fused = fddm.ddm(imgs, lags, mode="fft", precision=precision)._data
    monkeypatch.setenv("FDDM_B200_TEMPORAL_FUSED", "0")
    separate = fddm.ddm(imgs, lags, mode="fft", precision=precision)._data
    if precision == "ff":
        np.testing.assert_array_equal(fused, separate)
    elif precision == "f64":
        np.testing.assert_allclose(fused, separate, rtol=1e-11, atol=0.0)
    _check(fused, imgs, lags, "fft", precision, label=f"fused T={T}")
