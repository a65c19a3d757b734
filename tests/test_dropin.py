"""The reference's own front door with the b200 core bound in (CPU; needs the reference source tree).

Applies the two edits a FastDDM maintainer makes to bind the core (the
``'b200'`` rule in ``_fftopt.next_fast_len``, ``_backend['b200']`` in
``_ddm``) to the reference's Python package imported
in-process, then calls the reference's ``fastddm.ddm(..., core='b200')``.  The
device computation behind ``ddm_fft_b200`` / ``ddm_diff_b200`` is replaced by
the FP64 oracle (there is no GPU here), so what this checks is the boundary:
the arguments the reference's dispatch passes (``_ddm.py:169-190``), the array
the backend returns, and the container, axes and values the reference builds
from it, against the reference's own outputs on its test fixture.  The GPU
path itself is covered by the golden tests in test_ddm_gpu.py and
test_configs_gpu.py, which call the same backend functions.
"""

import sys
from pathlib import Path

import numpy as np
import pytest

import ddm_oracle as oracle

REF = Path("/root/reference")
pytestmark = pytest.mark.skipif(not (REF / "src" / "python" / "_ddm.py").exists(),
                                reason="the reference source tree is not present")


@pytest.fixture()
def bound_reference(monkeypatch):
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden

    # the reference package ("fastddm") and the stand-ins it gets for file readers are removed afterwards
    def ours(k):
        return k == "fastddm" or k.startswith("fastddm.") or k in ("tifffile", "skimage", "skimage.io", "nd2reader")

    before = {k: v for k, v in sys.modules.items() if ours(k)}
    mods = make_golden.import_reference(REF)
    ref_ddm, ref_fftopt = mods["_ddm"], mods["_fftopt"]

    import fastddm_gb300
    from fastddm_gb300 import _ddm_b200

    # edit 1 (src/python/_fftopt.py): 'b200' takes the cpp sizes
    orig = ref_fftopt.next_fast_len

    def next_fast_len(target, core="py", even=False):
        if core.upper() == "B200":
            return orig(target, "cpp")
        return orig(target, core) if not even else orig(target, core, even)

    monkeypatch.setattr(ref_fftopt, "next_fast_len", next_fast_len)
    monkeypatch.setattr(ref_ddm, "next_fast_len", next_fast_len)  # _ddm.py imports the name
    # edit 2 (src/python/_ddm.py): register the backend functions
    monkeypatch.setitem(ref_ddm._backend, "b200",
                        {"diff": fastddm_gb300.ddm_diff_b200, "fft": fastddm_gb300.ddm_fft_b200})

    calls = []

    def fake_device(img_seq, lags, nx, ny, nt, window=None, *, mode="fft", precision="ff", gpu_id=0,
                    host_out=False):
        """The oracle in place of the GPU: same arguments, same (device, host) result pair."""
        import torch

        calls.append({"shape": tuple(img_seq.shape), "lags": np.asarray(lags).copy(), "nx": nx, "ny": ny,
                      "nt": nt, "window": None if window is None else np.asarray(window).copy(), "mode": mode})
        w = None if window is None or np.size(window) == 0 else np.asarray(window)
        if mode == "fft":
            out = oracle.ddm_fft(np.asarray(img_seq), lags, nx, ny, nt, w)
        else:
            out = oracle.ddm_diff(np.asarray(img_seq), lags, nx, ny, w)
        host = torch.from_numpy(np.ascontiguousarray(out))
        return (host, host) if host_out else host

    monkeypatch.setattr(_ddm_b200, "ddm_device", fake_device)
    yield ref_ddm, calls
    for k in [k for k in sys.modules if ours(k)]:
        del sys.modules[k]
    sys.modules.update(before)


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_reference_front_door_dispatches_to_b200(bound_reference, golden, mode):
    ref_ddm, calls = bound_reference
    imgs, lags = golden["A_imgs"], golden["A_lags"]
    r = ref_ddm.ddm(imgs, lags, core="b200", mode=mode)
    assert len(calls) == 1
    c = calls[0]
    T, H, W = imgs.shape
    assert c["shape"] == (T, H, W) and c["mode"] == mode
    np.testing.assert_array_equal(c["lags"], lags)
    assert (c["nx"], c["ny"]) == (oracle.next_fast_len_cpp(W), oracle.next_fast_len_cpp(H))
    assert c["nt"] == (oracle.next_fast_len_cpp(2 * T) if mode == "fft" else 0)
    assert c["window"] is not None and c["window"].size == 0  # the reference passes an empty window
    # the reference's own container, axes and values around the b200 result
    assert type(r).__module__ == "fastddm.imagestructurefunction"
    np.testing.assert_array_equal(r.kx, golden["A_kx"])
    np.testing.assert_array_equal(r.ky, golden["A_ky"])
    assert r._data.shape == golden[f"A_{mode}"].shape
    assert oracle.rel_err(r._data, golden[f"A_{mode}"]) < 1e-10


def test_reference_front_door_window_and_errors(bound_reference, golden):
    ref_ddm, calls = bound_reference
    imgs, lags, win = golden["A_imgs"], golden["A_lags"], golden["A_window"]
    r = ref_ddm.ddm(imgs, lags, core="b200", mode="fft", window=win)
    np.testing.assert_array_equal(calls[-1]["window"], win)
    assert oracle.rel_err(r._data, golden["A_fft_win"]) < 1e-10
    with pytest.raises(RuntimeError, match="Window with shape"):
        ref_ddm.ddm(imgs, lags, core="b200", window=win[:-1])
    with pytest.raises(RuntimeError, match="Negative lags"):
        ref_ddm.ddm(imgs, [-1, 2], core="b200")
