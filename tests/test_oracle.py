"""The oracle and the host-side helpers against the reference's golden vectors (CPU only)."""

import numpy as np
import pytest

import ddm_oracle as oracle
import fastddm_gb300 as fddm

# The golden vectors come from the reference's FP64 `py` core; the reference's
# own cross-core tests accept `np.isclose` (rtol 1e-5).  The oracle restates
# the `cpp` core in FP64, so agreement is at FP64 rounding level.
ORACLE_RTOL = 1e-10


def _sizes(imgs, mode):
    T, H, W = imgs.shape
    nx, ny = oracle.next_fast_len_cpp(W), oracle.next_fast_len_cpp(H)
    return nx, ny, oracle.next_fast_len_cpp(2 * T)


@pytest.mark.parametrize("mode", ["fft", "diff"])
@pytest.mark.parametrize("case,winkey,outkey", [
    ("A", None, "A_{mode}"),
    ("A", "A_window", "A_{mode}_win"),
    ("B", "B_window", "B_{mode}"),
])
def test_oracle_matches_reference_core(golden, mode, case, winkey, outkey):
    imgs, lags = golden[f"{case}_imgs"], golden[f"{case}_lags"]
    nx, ny, nt = _sizes(imgs, mode)
    w = golden[winkey] if winkey else None
    out = oracle.ddm_fft(imgs, lags, nx, ny, nt, w) if mode == "fft" else oracle.ddm_diff(imgs, lags, nx, ny, w)
    ref = golden[outkey.format(mode=mode)]
    assert out.shape == ref.shape
    assert oracle.rel_err(out, ref) < ORACLE_RTOL
    assert np.isclose(out, ref).all()  # the reference test's own criterion


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_oracle_matches_reference_core_full_fixture(golden_confocal, mode):
    """The reference test's fixture uncropped (tests/test_ddm.py:14-16: 20 confocal frames of 256 x 256, lags 1..9)."""
    g = golden_confocal
    imgs, lags = g["C_imgs"], g["C_lags"]
    nx, ny, nt = _sizes(imgs, mode)
    out = oracle.ddm_fft(imgs, lags, nx, ny, nt) if mode == "fft" else oracle.ddm_diff(imgs, lags, nx, ny)
    ref = g[f"C_{mode}"]
    assert out.shape == ref.shape == (11, 256, 129)
    assert oracle.rel_err(out, ref) < ORACLE_RTOL
    assert np.isclose(out, ref).all()
    kx, ky = oracle.axes(nx, ny)
    np.testing.assert_array_equal(kx, g["C_kx"])
    np.testing.assert_array_equal(ky, g["C_ky"])


def test_sampled_exact_matches_full_exact(golden):
    """The sampled direct-DFT yardstick (used at full sizes) equals the extended-precision one on its columns."""
    imgs, lags, w = golden["B_imgs"], golden["B_lags"], golden["B_window"]
    nx, ny, _ = _sizes(imgs, "fft")
    cols = [0, 1, 4, nx // 2]
    full = oracle.ddm_exact(imgs, lags, nx, ny, w)
    assert oracle.rel_err(oracle.sampled_exact(imgs, lags, nx, ny, cols, w), full[:, :, cols]) < 1e-11


def test_oracle_fft_vs_diff_agree(golden):
    imgs, lags = golden["A_imgs"], golden["A_lags"]
    nx, ny, nt = _sizes(imgs, "fft")
    a = oracle.ddm_fft(imgs, lags, nx, ny, nt)
    b = oracle.ddm_diff(imgs, lags, nx, ny)
    assert oracle.rel_err(a, b) < 1e-9


def test_oracle_detects_a_planted_error(golden):
    """A wrong normalisation planted in the oracle must be caught by the same check."""
    imgs, lags = golden["A_imgs"], golden["A_lags"]
    nx, ny, nt = _sizes(imgs, "fft")
    bad = oracle.ddm_fft(imgs, lags, nx, ny, nt)
    bad[0] *= 1 + 1e-7
    assert oracle.rel_err(bad, golden["A_fft"]) > ORACLE_RTOL


def test_axes_match_reference(golden):
    for case in ("A", "B"):
        imgs = golden[f"{case}_imgs"]
        nx, ny, _ = _sizes(imgs, "fft")
        kx, ky = oracle.axes(nx, ny)
        np.testing.assert_array_equal(kx, golden[f"{case}_kx"])
        np.testing.assert_array_equal(ky, golden[f"{case}_ky"])


def test_next_fast_len_tables(golden):
    targets = np.arange(1, 3001)
    np.testing.assert_array_equal([oracle.next_fast_len_cpp(int(t)) for t in targets], golden["nfl_cpp"])
    np.testing.assert_array_equal([fddm.next_fast_len(int(t), "cpp") for t in targets], golden["nfl_cpp"])
    np.testing.assert_array_equal([fddm.next_fast_len(int(t), "b200") for t in targets], golden["nfl_cpp"])
    np.testing.assert_array_equal([fddm.next_fast_len(int(t), "cuda") for t in targets], golden["nfl_cuda"])
    np.testing.assert_array_equal([fddm.next_fast_len(int(t), "cuda", True) for t in targets], golden["nfl_cuda_even"])
    with pytest.raises(ValueError):
        fddm.next_fast_len(1000, "opencl")


def test_lags_helpers(golden):
    for key in [k for k in golden if k.startswith("logspace_")]:
        _, stop, num, ep = key.split("_")
        np.testing.assert_array_equal(fddm.lags.logspace_int(int(stop), num=int(num), endpoint=bool(int(ep))), golden[key])
    np.testing.assert_array_equal(fddm.lags.fibonacci(13, endpoint=True), golden["fib_13_1"])
    np.testing.assert_array_equal(fddm.lags.fibonacci(100), golden["fib_100_0"])


def test_windows_bit_identical(golden):
    for shape in ((5, 7), (16, 16), (3, 24, 9)):
        key = "x".join(map(str, shape))
        np.testing.assert_array_equal(fddm.window.blackman(shape), golden[f"win_blackman_{key}"])
        np.testing.assert_array_equal(fddm.window.blackman_harris(shape), golden[f"win_bh_{key}"])
    np.testing.assert_array_equal(fddm.window.blackman_harris(golden["A_imgs"].shape), golden["A_window"])


def test_masks(golden):
    np.testing.assert_array_equal(fddm.mask.central_cross_mask((48, 17)), golden["ccm_48x17"])
    kx = 2 * np.pi * np.fft.fftfreq(16)[:9]
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(12))
    np.testing.assert_array_equal(fddm.mask.central_cross_mask((12, 9), kx, ky), golden["ccm_k_12x9"])


@pytest.mark.parametrize("tag", ["A_aa", "A_aa_edges", "A_aa_w"])
def test_oracle_azimuthal_average(golden, tag):
    data = golden["A_fft"]
    kx, ky = golden["A_kx"], golden["A_ky"]
    width = 2 * (len(kx) - 1)
    if tag == "A_aa":
        args = dict(bins=len(ky) // 2, rng=(0, ky[-1]), mask=fddm.mask.central_cross_mask(data.shape[1:]))
    elif tag == "A_aa_edges":
        args = dict(bins=np.linspace(0, ky[-1], num=len(ky) // 2).tolist(), mask=fddm.mask.central_cross_mask(data.shape[1:]))
    else:
        args = dict(bins=7, weights=golden["A_aa_w_weights"])
    avg, err, k, edges = oracle.azimuthal_average(data, kx, ky, width, **args)
    np.testing.assert_array_equal(avg, golden[f"{tag}_data"])
    np.testing.assert_array_equal(err, golden[f"{tag}_err"])
    np.testing.assert_array_equal(k, golden[f"{tag}_k"])
    np.testing.assert_array_equal(edges, golden[f"{tag}_edges"])


@pytest.mark.parametrize("tag", ["A_aa", "A_aa_edges", "A_aa_w"])
def test_host_bin_setup_bit_identical(golden, tag):
    """The host half of the b200 azimuthal average (edges, masking, k per bin)."""
    from fastddm_gb300.azimuthalaverage import bin_setup

    data = golden["A_fft"]
    kx, ky = golden["A_kx"], golden["A_ky"]
    counts = np.full(data.shape[1:], 2)
    counts[:, 0] = 1
    counts[:, -1] = 1
    X, Y = np.meshgrid(kx, ky)
    dist = np.sqrt(X ** 2 + Y ** 2)
    mask = fddm.mask.central_cross_mask(data.shape[1:])
    if tag == "A_aa":
        s = bin_setup(dist, len(ky) // 2, (0, ky[-1]), mask, None, counts, True)
    elif tag == "A_aa_edges":
        s = bin_setup(dist, np.linspace(0, ky[-1], num=len(ky) // 2).tolist(), None, mask, None, counts, True)
    else:
        s = bin_setup(dist, 7, None, None, golden["A_aa_w_weights"], counts, True)
    np.testing.assert_array_equal(s.k, golden[f"{tag}_k"])
    np.testing.assert_array_equal(s.bin_edges, golden[f"{tag}_edges"])


@pytest.mark.parametrize("shape,bins", [((24, 13), 7), ((33, 17), 12), ((16, 9), [0.0, 0.5, 1.0, 1.7, 2.9])])
def test_azimuthal_binning_host_side_matches_loops(shape, bins):
    """The host half of ``azimuthal_average`` (edges, pixel selection, per-bin weight sums
    and the mean |k| of every bin) equals the reference's pixel loops bit for bit,
    including empty bins, masked pixels and zero weights."""
    from fastddm_gb300.azimuthalaverage import bin_setup

    rng = np.random.default_rng(sum(shape))
    ky = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(shape[0]))
    kx = 2 * np.pi * np.fft.fftfreq(2 * (shape[1] - 1))[: shape[1]]
    X, Y = np.meshgrid(kx, ky)
    dist = np.sqrt(X ** 2 + Y ** 2)
    mask = rng.random(shape) > 0.2
    weights = rng.random(shape) * (rng.random(shape) > 0.1)
    counts = np.full(shape, 2.0)
    counts[:, 0] = 1
    data = rng.random((3,) + shape)
    for m, w in ((None, None), (mask, None), (mask, weights)):
        setup = bin_setup(dist, bins, None, m, w, counts, True)
        _, _, x, edges = oracle.azimuthal_average_array(data, dist, bins, None, m, w, counts, True)
        np.testing.assert_array_equal(setup.bin_edges, edges)
        np.testing.assert_array_equal(setup.k, x)
