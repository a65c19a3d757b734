"""``.sf.ddm`` written from device memory (streamed through pinned staging
buffers) against the same file written from host memory (needs a GPU)."""

import numpy as np
import pytest

from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]


def test_device_stream_equals_host_write(built_lib, tmp_path):
    import torch

    from fastddm_gb300 import _io

    # two full 32 MiB staging chunks and a ragged third
    L, ny, nkx = 80, 256, 129 * 4 + 7
    g = torch.Generator(device="cuda").manual_seed(3)
    dev = torch.randn((L + 2, ny, nkx), dtype=torch.float64, device="cuda", generator=g)
    assert dev.numel() * 8 > 2 * 32 * 2**20
    kx = np.linspace(0, np.pi, nkx)
    ky = np.linspace(-np.pi, np.pi, ny, endpoint=False)
    tau = np.arange(1, L + 1, dtype=np.float64)
    for _ in range(2):  # the staging buffers are reused on the second call
        _io.sf_write(str(tmp_path / "dev.sf.ddm"), dev, kx, ky, tau, 2 * (nkx - 1), ny, 0.5, 0.1)
    _io.sf_write(str(tmp_path / "host.sf.ddm"), dev.cpu().numpy(), kx, ky, tau, 2 * (nkx - 1), ny, 0.5, 0.1)
    assert (tmp_path / "dev.sf.ddm").read_bytes() == (tmp_path / "host.sf.ddm").read_bytes()


def test_ddm_save_equals_object_save(built_lib, tmp_path):
    import fastddm_gb300 as fddm

    rng = np.random.default_rng(5)
    imgs = rng.poisson(200.0, size=(40, 48, 64)).astype(np.uint16)
    lags = [1, 2, 5, 13, 39]
    w = fddm.window.blackman_harris((48, 64))
    r = fddm.ddm(imgs, lags, window=w)
    r.save(str(tmp_path / "host"))
    r.save(str(tmp_path / "dev"), from_device=True)
    path = fddm.ddm_save(imgs, lags, str(tmp_path / "direct"), window=w)
    ref = (tmp_path / "host.sf.ddm").read_bytes()
    assert (tmp_path / "dev.sf.ddm").read_bytes() == ref
    assert open(path, "rb").read() == ref
    back = fddm.load(path)
    np.testing.assert_array_equal(back._data, r._data)
    np.testing.assert_array_equal(back.tau, r.tau)


def test_tiff_ingest_pinned_into_ddm(built_lib, tmp_path):
    """A TIFF stack decoded into page-locked memory goes through ddm like any array."""
    import fastddm_gb300 as fddm
    from fastddm_gb300 import utils
    from tiffgen import write_tiff

    rng = np.random.default_rng(9)
    frames = rng.poisson(300.0, size=(48, 40, 56)).astype(np.uint16)
    p = tmp_path / "stack.tif"
    write_tiff(p, frames, rows_per_strip=7, compression="lzw", predictor=True)
    pinned = utils.read_images(str(p), pinned=True)
    np.testing.assert_array_equal(pinned, frames)
    a = fddm.ddm(pinned, [1, 3, 20])._data
    b = fddm.ddm(frames, [1, 3, 20])._data
    np.testing.assert_array_equal(a, b)
