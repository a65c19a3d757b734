"""``.sf.ddm`` / ``.aa.ddm`` files against the reference's own writers (CPU).

The fixtures ``tests/golden/golden_*.ddm`` were written by the reference's
``SFWriter`` and ``AAWriter`` (``tests/golden/make_golden_files.py``).  This
package must write the same bytes and read those files back.
"""

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _golden_sf(golden):
    from fastddm_gb300 import ImageStructureFunction

    tau = np.arange(1, 10, dtype=np.float64)
    return ImageStructureFunction(golden["A_fft"].copy(), golden["A_kx"], golden["A_ky"], 32, 48, tau, 0.65, 0.05)


def test_sf_writer_matches_reference_bytes(built_lib, golden, tmp_path):
    sf = _golden_sf(golden)
    sf.save(str(tmp_path / "out"))  # suffix appended as the reference does
    assert (tmp_path / "out.sf.ddm").read_bytes() == (GOLDEN / "golden_sf.sf.ddm").read_bytes()
    # a name that already ends in .sf.ddm, in a directory that does not exist yet
    sf.save(str(tmp_path / "sub" / "dir" / "x.sf.ddm"))
    assert (tmp_path / "sub" / "dir" / "x.sf.ddm").read_bytes() == (GOLDEN / "golden_sf.sf.ddm").read_bytes()


def test_sf_reader_reads_reference_file(golden):
    from fastddm_gb300 import SFReader, load

    sf = _golden_sf(golden)
    with SFReader(str(GOLDEN / "golden_sf.sf.ddm")) as r:
        obj = r.load()
        np.testing.assert_array_equal(obj._data, sf._data)
        np.testing.assert_array_equal(r.get_kx(False), sf.kx)
        np.testing.assert_array_equal(r.get_kx(True), sf.full_kx())
        np.testing.assert_array_equal(r.get_ky(), sf.ky)
        np.testing.assert_array_equal(r.get_tau(), sf.tau)
        for i in (0, 4, 8):
            np.testing.assert_array_equal(r.get_frame(i), sf.full_slice(i))
            np.testing.assert_array_equal(r.get_frame(i, full=False), sf.data[i])
        np.testing.assert_array_equal(r.get_power_spec(), sf.full_power_spec())
        np.testing.assert_array_equal(r.get_var(full=False), sf.var)
        with pytest.raises(IndexError):
            r.get_frame(9)
    assert (obj.width, obj.height, obj.pixel_size, obj.delta_t) == (32, 48, 0.65, 0.05)
    obj2 = load(str(GOLDEN / "golden_sf.sf.ddm"))
    np.testing.assert_array_equal(obj2._data, sf._data)


@pytest.mark.parametrize("name", ["golden_aa.aa.ddm", "golden_aa_noerr.aa.ddm"])
def test_aa_round_trip_matches_reference_bytes(name, tmp_path):
    from fastddm_gb300 import AAReader, load

    ref = (GOLDEN / name).read_bytes()
    with AAReader(str(GOLDEN / name)) as r:
        avg = r.load()
        k0 = r.get_k_slice(0)
        e0 = r.get_k_slice_err(0)
        with pytest.raises(IndexError):
            r.get_k_slice(len(avg.k))
    np.testing.assert_array_equal(k0, avg.data[0])
    if avg._err is None:
        assert e0 is None
    else:
        np.testing.assert_array_equal(e0, avg.err[0])
    avg.save(str(tmp_path / "aa"))
    assert (tmp_path / "aa.aa.ddm").read_bytes() == ref
    again = load(str(tmp_path / "aa.aa.ddm"))
    np.testing.assert_array_equal(again._data, avg._data)


def test_aa_values_match_golden_average(golden):
    """The reference's average in the file is the one the golden fixture holds (bins=5 is not
    in golden.npz, but the error-free file's rows are a prefix of the full one)."""
    from fastddm_gb300 import load

    full = load(str(GOLDEN / "golden_aa.aa.ddm"))
    part = load(str(GOLDEN / "golden_aa_noerr.aa.ddm"))
    np.testing.assert_array_equal(part._data, full._data[:4])
    assert part._err is None and full._err is not None
    np.testing.assert_array_equal(full.tau, np.arange(1, 10))


def test_file_errors(tmp_path):
    from fastddm_gb300 import AAReader, SFReader, load

    with pytest.raises(RuntimeError, match="extension"):
        load(str(tmp_path / "x.fit.ddm"))
    # an .aa.ddm file is not an image structure function file
    bad = tmp_path / "wrong.sf.ddm"
    bad.write_bytes((GOLDEN / "golden_aa.aa.ddm").read_bytes())
    with pytest.raises(RuntimeError, match="identifier 22"):
        SFReader(str(bad))
    junk = tmp_path / "junk.aa.ddm"
    junk.write_bytes(b"XX" + bytes(100))
    with pytest.raises(RuntimeError, match="Byteorder"):
        AAReader(str(junk))


def test_sf_writer_reports_io_errors(built_lib, golden, tmp_path):
    from fastddm_gb300 import _io
    from fastddm_gb300._lib import FddmError

    sf = _golden_sf(golden)
    d = tmp_path / "a_directory"
    d.mkdir()
    with pytest.raises(FddmError, match="cannot open"):
        _io.sf_write(str(d), sf._data, sf.kx, sf.ky, sf.tau, 32, 48)
    with pytest.raises(ValueError):
        _io.sf_write(str(tmp_path / "y.sf.ddm"), sf._data, sf.kx[:-1], sf.ky, sf.tau, 32, 48)
