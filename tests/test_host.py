"""Host-side logic of the b200 core: front-door validation, containers, C ABI exports (CPU only)."""

import ctypes
import re
import warnings
from pathlib import Path

import numpy as np
import pytest

import fastddm_gb300 as fddm
from fastddm_gb300.imagestructurefunction import ImageStructureFunction, _reconstruct_full_spectrum

ROOT = Path(__file__).resolve().parent.parent
IMGS = np.zeros((5, 8, 6), dtype=np.uint16)


def test_unknown_core_and_mode():
    with pytest.raises(RuntimeError, match="Unknown core"):
        fddm.ddm(IMGS, [1], core="cuda")
    with pytest.raises(RuntimeError, match="Unknown mode"):
        fddm.ddm(IMGS, [1], mode="fast")


def test_lag_errors():
    with pytest.raises(RuntimeError, match="Negative lags"):
        fddm.ddm(IMGS, [-1], mode="diff")
    with pytest.raises(RuntimeError, match="Lags larger"):
        fddm.ddm(IMGS, [5])


def test_window_shape_error():
    with pytest.raises(RuntimeError, match="incompatible"):
        fddm.ddm(IMGS, [1, 2], window=np.ones((9, 6)))


def test_backend_registry_matches_reference_keys():
    assert set(fddm._backend["b200"]) == {"fft", "diff"}


def test_isf_views_and_full_plane(golden):
    data = golden["A_fft"]
    kx, ky = golden["A_kx"], golden["A_ky"]
    isf = ImageStructureFunction(data.copy(), kx.copy(), ky.copy(), 32, 48, np.arange(1.0, 10.0))
    assert isf.shape == (9, 48, 17)
    assert len(isf) == 9
    np.testing.assert_array_equal(isf.power_spec, data[-2])
    np.testing.assert_array_equal(isf.var, data[-1])
    assert isf.full_shape() == (9, 48, 32)
    # full plane of a real image's power spectrum: Hermitian symmetry |F(-k)| = |F(k)|
    full = isf.full_power_spec()
    assert full.shape == (48, 32)
    np.testing.assert_allclose(full[1:, 1:], full[1:, 1:][::-1, ::-1], rtol=1e-12)
    fk = isf.full_kx()
    np.testing.assert_allclose(fk, 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(32)))
    isf.delta_t = 0.5
    np.testing.assert_allclose(isf.tau, 0.5 * np.arange(1.0, 10.0))
    with pytest.raises(IndexError):
        isf.full_slice(9)


@pytest.mark.parametrize("shape", [(6, 4), (6, 5), (7, 4), (7, 5)])
def test_full_plane_reconstruction_matches_fft2(shape):
    """Half plane -> full plane equals fftshift(|fft2|^2) of a real image."""
    rng = np.random.default_rng(0)
    img = rng.standard_normal(shape)
    full = np.abs(np.fft.fft2(img)) ** 2
    half = np.fft.fftshift(np.abs(np.fft.rfft2(img)) ** 2, axes=0)
    rec = _reconstruct_full_spectrum(half, shape)
    np.testing.assert_allclose(rec, np.fft.fftshift(full), rtol=1e-12)


def _declared_symbols():
    text = (ROOT / "include" / "fddm_b200.h").read_text()
    return sorted(set(re.findall(r"\b(fddm_b200_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    syms = _declared_symbols()
    assert len(syms) >= 6
    for s in syms:
        assert hasattr(built_lib, s), s
    # pure host calls only (no device work on the CPU)
    assert built_lib.fddm_b200_version() >= 100


def test_workspace_query_and_errors(built_lib):
    from fastddm_gb300 import _lib

    size = ctypes.c_size_t(0)
    # fft mode, config of 64 frames of 128 x 128
    rc = built_lib.fddm_b200_workspace_size(0, 0, 64, 128, 128, 63, 128, 128, 128, 0, ctypes.byref(size))
    assert rc == 0
    assert size.value >= 65 * 128 * 64 * 16
    # nt too short for the sequence
    rc = built_lib.fddm_b200_workspace_size(0, 0, 64, 128, 128, 63, 128, 128, 100, 0, ctypes.byref(size))
    assert rc == _lib.FDDM_ERR_UNSUPPORTED
    assert b"nt" in built_lib.fddm_b200_last_error()
    # a size with a prime factor the kernels do not handle
    rc = built_lib.fddm_b200_workspace_size(1, 0, 8, 17, 17, 3, 17, 17, 0, 0, ctypes.byref(size))
    assert rc == _lib.FDDM_ERR_UNSUPPORTED
    assert b"17" in built_lib.fddm_b200_last_error()
    # unknown precision
    rc = built_lib.fddm_b200_workspace_size(0, 9, 8, 16, 16, 3, 16, 16, 16, 0, ctypes.byref(size))
    assert rc == _lib.FDDM_ERR_INVALID
    # null pointers are rejected without touching the device
    rc = built_lib.fddm_b200_ddm_fft(None, 0, 8, 16, 16, None, 0, 16, 16, 16, None, None, None, 0, 0, None)
    assert rc == _lib.FDDM_ERR_INVALID


def test_fft_lags_must_increase(built_lib):
    """fft mode refuses non-increasing lags before any device work (the arguments are
    checked on the host, so dummy device pointers are never touched)."""
    from fastddm_gb300 import _lib

    dummy = ctypes.c_void_p(256)
    for lags in ([5, 1, 3], [1, 3, 3]):
        arr = (ctypes.c_uint32 * len(lags))(*lags)
        rc = built_lib.fddm_b200_ddm_fft(dummy, 0, 8, 16, 16, arr, len(lags), 16, 16, 16, None, dummy, dummy,
                                         1 << 20, 0, None)
        assert rc == _lib.FDDM_ERR_INVALID
        assert b"strictly increasing" in built_lib.fddm_b200_last_error()


def test_status_to_exception(built_lib):
    from fastddm_gb300 import _lib

    with pytest.raises(_lib.FddmError):
        _lib.check(_lib.FDDM_ERR_INVALID)
    with pytest.raises(_lib.FddmError, match="Not enough memory"):
        _lib.check(_lib.FDDM_ERR_NOMEM)


def test_lag_zero_warning_before_device():
    """Lag 0 is dropped with a warning (the reference's behaviour) before any device call."""
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        try:
            fddm.ddm(IMGS, [0, 1])
        except RuntimeError:
            pass  # no GPU in this process
    assert any("Found 0 in lags" in str(x.message) for x in w)


def test_bindings_match_the_header_declarations():
    """Every ctypes binding has as many arguments as its C declaration: a missing one would send the
    trailing arguments (the stream) through ctypes' default int conversion."""
    import re

    from fastddm_gb300 import _lib

    text = (ROOT / "include" / "fddm_b200.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    decls = {}
    for m in re.finditer(r"\b(fddm_b200_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = " ".join(m.group(2).split())
        decls[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    for name, (_, argtypes) in _lib._SIGNATURES.items():
        assert name in decls, name
        assert len(argtypes) == decls[name], (name, len(argtypes), decls[name])
