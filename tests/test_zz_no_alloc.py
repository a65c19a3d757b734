"""The allocation-free fft-mode entry point (needs a GPU).

fddm_b200_ddm_fft_noalloc serves callers that cannot allocate device memory
when they need a result (an acquisition callback, a plugin whose host owns all
device memory): its scratch is a fixed 64 MiB array inside the library.  It
must give the same structure function as fddm_b200_ddm_fft with a caller
workspace, call after call, since every call reuses the array the previous one
left behind.  Collected last on purpose, so a failure here comes after every
other test has run.
"""

import ctypes

import numpy as np
import pytest

from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]

# the float-float tier tolerance of the other parity tests
RTOL = 1e-8


def _frames(shape, seed):
    rng = np.random.default_rng(seed)
    T, H, W = shape
    yy, xx = np.mgrid[0:H, 0:W]
    out = []
    for t in range(T):
        scene = 200.0 + 1500.0 * np.exp(-((xx - 0.3 * W - 0.2 * t) ** 2 + (yy - 0.5 * H) ** 2) / 30.0)
        out.append(rng.poisson(scene))
    return np.stack(out).astype(np.uint16)


PREC = {"ff": 0, "f64": 1, "f32": 2}


def _run_pair(lib, torch, imgs, lags, window, precision="ff", calls=2):
    from fastddm_gb300 import _lib
    from fastddm_gb300._fftopt import next_fast_len

    T, H, W = imgs.shape
    nx, ny, nt = next_fast_len(W, "b200"), next_fast_len(H, "b200"), next_fast_len(2 * T, "b200")
    dev = torch.device("cuda", 0)
    frames = torch.from_numpy(imgs.astype(np.int32)).to(torch.int16 if imgs.max() < 32768 else torch.int32).to(dev)
    code = 1 if frames.dtype == torch.int16 else 3
    win = torch.from_numpy(window).to(dev) if window is not None else None
    wptr = win.data_ptr() if win is not None else None
    lags_c = np.ascontiguousarray(lags, dtype=np.uint32)
    lp = lags_c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    shape = (len(lags_c) + 2, ny, nx // 2 + 1)
    stream = torch.cuda.current_stream(dev).cuda_stream

    size = ctypes.c_size_t()
    prec = PREC[precision]
    _lib.check(lib.fddm_b200_workspace_size(0, prec, T, H, W, len(lags_c), nx, ny, nt, int(win is not None),
                                            ctypes.byref(size)))
    work = torch.empty(size.value, dtype=torch.uint8, device=dev)
    ref = torch.empty(shape, dtype=torch.float64, device=dev)
    _lib.check(lib.fddm_b200_ddm_fft(frames.data_ptr(), code, T, H, W, lp, len(lags_c), nx, ny, nt, wptr,
                                     ref.data_ptr(), work.data_ptr(), size.value, prec, stream))
    outs = []
    for _ in range(calls):  # calls in a row share the static scratch
        out = torch.full(shape, float("nan"), dtype=torch.float64, device=dev)
        _lib.check(lib.fddm_b200_ddm_fft_noalloc(frames.data_ptr(), code, T, H, W, lp, len(lags_c), nx, ny, nt,
                                                 wptr, out.data_ptr(), prec, stream))
        outs.append(out.cpu().numpy())
    return ref.cpu().numpy(), outs, size.value


@pytest.mark.parametrize("shape,lags,windowed", [
    ((40, 48, 64), [1, 2, 3, 5, 8, 13, 21, 39], False),
    ((64, 128, 128), list(range(1, 64)), True),
])
def test_noalloc_matches_workspace_entry_point(built_lib, shape, lags, windowed):
    torch = pytest.importorskip("torch")
    from fastddm_gb300.window import blackman_harris

    imgs = _frames(shape, seed=shape[0])
    window = blackman_harris(shape) if windowed else None
    ref, outs, _ = _run_pair(built_lib, torch, imgs, lags, window)
    for out in outs:
        assert np.all(np.isfinite(out))
        np.testing.assert_allclose(out, ref, rtol=RTOL, atol=0.0)


def test_noalloc_shrinks_its_frame_chunk_and_alternates_problems(built_lib):
    """A problem whose workspace (at the full frame chunk) exceeds the 64 MiB array but fits once the
    frame chunk shrinks, alternated with another shape and tier: each call starts from the array the
    previous, different problem left behind, and must still equal its workspace twin."""
    torch = pytest.importorskip("torch")

    small = _frames((40, 48, 64), seed=40)
    big = _frames((520, 128, 128), seed=520)  # FP32 tier: ~74 MiB of workspace at the full chunk
    for imgs, lags, precision in ((small, [1, 2, 3, 5, 8, 13, 21, 39], "ff"),
                                  (big, list(range(1, 520)), "f32"),
                                  (small, [1, 2, 3, 5, 8, 13, 21, 39], "ff"),
                                  (big, list(range(1, 520)), "f32")):
        ref, outs, need = _run_pair(built_lib, torch, imgs, lags, None, precision, calls=1)
        if imgs is big:
            assert need > 64 << 20  # only the shrunken frame chunk fits the static scratch
        for out in outs:
            assert np.all(np.isfinite(out))
            np.testing.assert_allclose(out, ref, rtol=RTOL, atol=0.0)


def test_noalloc_rejects_problems_beyond_its_scratch(built_lib):
    """A stack whose workspace exceeds the 64 MiB array is refused before any device work."""
    torch = pytest.importorskip("torch")
    from fastddm_gb300 import _lib

    dev = torch.device("cuda", 0)
    dummy_in = torch.zeros(16, dtype=torch.uint8, device=dev)
    dummy_out = torch.zeros(16, dtype=torch.float64, device=dev)
    lags = np.arange(1, 100, dtype=np.uint32)
    lp = lags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    # 1000 frames of 512 x 512: the spectrum alone needs about 2 GB
    rc = built_lib.fddm_b200_ddm_fft_noalloc(dummy_in.data_ptr(), 0, 1000, 512, 512, lp, len(lags), 512, 512, 2000,
                                             None, dummy_out.data_ptr(), 0, None)
    assert rc == _lib.FDDM_ERR_NOMEM
    msg = built_lib.fddm_b200_last_error().decode()
    assert "static scratch" in msg and "bytes" in msg
