"""TIFF ingest (``fastddm_gb300.utils``, ``fddm_b200_tiff_*``) on the CPU.

Files are written by ``tests/tiffgen.py`` in every layout the native reader
supports: both byte orders, classic and BigTIFF, one or many strips,
uncompressed, PackBits and LZW with and without the horizontal predictor,
every sample type.  The decoded frames must equal the arrays written.
"""

import numpy as np
import pytest

from tiffgen import lzw, packbits, write_tiff

DTYPES = ["uint8", "uint16", "int16", "uint32", "int32", "float32", "float64", "uint64", "int64"]


def _frames(dtype, n=3, h=37, w=29, seed=0):
    rng = np.random.default_rng(seed)
    if np.dtype(dtype).kind == "f":
        return rng.normal(100.0, 30.0, size=(n, h, w)).astype(dtype)
    info = np.iinfo(dtype)
    lo, hi = max(info.min, -30000), min(info.max, 60000)
    a = rng.integers(lo, hi, size=(n, h, w))
    a[:, :5, :] = a[:, :1, :1]  # long runs for the compressors
    return a.astype(dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("byteorder", ["<", ">"])
def test_uncompressed_all_types(built_lib, tmp_path, dtype, byteorder):
    from fastddm_gb300 import utils

    frames = _frames(dtype)
    p = tmp_path / "s.tif"
    write_tiff(p, frames, byteorder=byteorder, rows_per_strip=8)
    n, h, w, dt = utils.tiff_info(str(p))
    assert (n, h, w, np.dtype(dt)) == (3, 37, 29, np.dtype(dtype))
    np.testing.assert_array_equal(utils.read_images(str(p)), frames)


@pytest.mark.parametrize("compression,predictor", [("packbits", False), ("lzw", False), ("lzw", True)])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "int32"])
@pytest.mark.parametrize("bigtiff", [False, True])
def test_compressed(built_lib, tmp_path, compression, predictor, dtype, bigtiff):
    from fastddm_gb300 import utils

    frames = _frames(dtype, n=4, seed=7)
    p = tmp_path / "c.tif"
    write_tiff(p, frames, byteorder=">" if bigtiff else "<", bigtiff=bigtiff, rows_per_strip=10,
               compression=compression, predictor=predictor)
    np.testing.assert_array_equal(utils.tiff2numpy(str(p)), frames)


def test_lzw_long_strip_resets_table(built_lib, tmp_path):
    """A strip long enough to fill the 4096-entry table (clear codes mid-strip)."""
    from fastddm_gb300 import utils

    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, size=(1, 160, 200)).astype(np.uint8)
    assert len(lzw(img.tobytes())) > 6000
    p = tmp_path / "big.tif"
    write_tiff(p, img, compression="lzw")
    np.testing.assert_array_equal(utils.read_images(str(p)), img[0])


def test_packbits_round_trip_helper():
    data = bytes([1, 1, 1, 2, 3, 4, 4]) + bytes(300) + bytes(range(200))
    # the test encoder itself: decoded by the textbook rule
    enc, out, i = packbits(data), bytearray(), 0
    while i < len(enc):
        c = enc[i] if enc[i] < 128 else enc[i] - 256
        i += 1
        if c >= 0:
            out += enc[i:i + c + 1]
            i += c + 1
        elif c != -128:
            out += bytes([enc[i]]) * (1 - c)
            i += 1
    assert bytes(out) == data


def test_page_selection_and_single_page(built_lib, tmp_path):
    from fastddm_gb300 import utils

    frames = _frames("uint16", n=6)
    p = tmp_path / "m.tif"
    write_tiff(p, frames)
    np.testing.assert_array_equal(utils.read_images(str(p), seq=range(1, 5)), frames[1:5])
    np.testing.assert_array_equal(utils.read_images(str(p), seq=[5, 0, -1]), frames[[5, 0, 5]])
    with pytest.raises(IndexError):
        utils.read_images(str(p), seq=[6])
    one = tmp_path / "one.tif"
    write_tiff(one, frames[:1])
    assert utils.read_images(str(one)).shape == (37, 29)  # one image, as tifffile returns it


def test_list_of_files(built_lib, tmp_path):
    from fastddm_gb300 import utils

    frames = _frames("uint8", n=5)
    names = []
    for i, f in enumerate(frames):
        names.append(str(tmp_path / f"img_{i:03d}.tif"))
        write_tiff(names[-1], [f], byteorder="<>"[i % 2], compression=["none", "lzw", "packbits"][i % 3])
    np.testing.assert_array_equal(utils.read_images(names), frames)
    write_tiff(tmp_path / "odd.tif", [frames[0][:10]])
    with pytest.raises(RuntimeError, match="differs"):
        utils.read_images(names + [str(tmp_path / "odd.tif")])


def test_errors(built_lib, tmp_path):
    from fastddm_gb300 import utils
    from fastddm_gb300._lib import FddmError

    bad = tmp_path / "x.tif"
    bad.write_bytes(b"not a tiff at all")
    with pytest.raises(FddmError, match="not a TIFF"):
        utils.read_images(str(bad))
    with pytest.raises(FddmError, match="cannot open"):
        utils.read_images(str(tmp_path / "missing.tif"))
    with pytest.raises(RuntimeError, match="Failed to open"):
        utils.read_images(42)
    with pytest.raises(NotImplementedError):
        utils.read_images(str(bad), color_seq=[0])  # colour stacks need tifffile
    # truncated strip data
    frames = _frames("uint16", n=2)
    good = tmp_path / "t.tif"
    write_tiff(good, frames)
    raw = good.read_bytes()
    cut = tmp_path / "cut.tif"
    cut.write_bytes(raw[:200] + bytes(len(raw) - 200))  # IFDs zeroed: no pages
    with pytest.raises(FddmError):
        utils.read_images(str(cut))
