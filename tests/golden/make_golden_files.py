"""Generate the binary file fixtures ``golden_sf.sf.ddm`` and ``golden_aa.aa.ddm``
with the reference's own writers.

The reference's ``SFWriter`` (``src/python/imagestructurefunction.py:409-627``)
and ``AAWriter`` (``src/python/azimuthalaverage.py:567-753``) are imported from
the reference source tree (as ``make_golden.py`` does) and write a small image
structure function (the reference fixture's structure function from
``golden.npz``, case A without window) and its azimuthal average.  The tests
check that this package writes the same bytes and reads these files back.

Usage (needs the reference checkout; the files it writes are committed):

    python tests/golden/make_golden_files.py /path/to/fastddm-reference
"""

from __future__ import annotations

import importlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import import_reference  # noqa: E402


def main(root: Path) -> None:
    import_reference(root)
    isf = importlib.import_module("fastddm.imagestructurefunction")
    aa = importlib.import_module("fastddm.azimuthalaverage")
    g = np.load(HERE / "golden.npz")
    data = np.ascontiguousarray(g["A_fft"])  # (L + 2, ny, nkx) = (11, 48, 17), frames 48 x 32
    L = data.shape[0] - 2
    tau = np.arange(1, L + 1, dtype=np.float64)
    sf = isf.ImageStructureFunction(data, g["A_kx"], g["A_ky"], 32, 48, tau, 0.65, 0.05)
    sf.save(str(HERE / "golden_sf"))
    # azimuthal average of the same object: the reference's own routine
    avg = aa.azimuthal_average(sf, bins=5, range=None, eval_err=True)
    avg.save(str(HERE / "golden_aa"))
    # the reference's eval_err=False path stops with an UnboundLocalError
    # (azimuthalaverage.py:438), so the error-free file is written from a
    # container built directly
    avg_noerr = aa.AzimuthalAverage(avg._data[:4].copy(), None, avg.k[:4].copy(), avg.tau.copy(), avg.bin_edges[:4].copy())
    avg_noerr.save(str(HERE / "golden_aa_noerr"))
    print("wrote", sorted(p.name for p in HERE.glob("golden_*.ddm")))


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
