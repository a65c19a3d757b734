"""Autotuner of the temporal kernels' launch shape, and its committed table.

The temporal stage's launch shape (CTA size 128/256/512 threads; the needed
prefix sums and per-lag tables in shared memory or in global scratch) decides
how many independent CTAs share an SM, which moves the stage's time by up to
2x for series of a few hundred to a few thousand frames.  The library picks
it per problem class (precision, mode, number of frames, number of lags):

* from its tuning table, which this module fills at import from the committed
  ``tuning_table.json`` (measured on a GB300 by :func:`tune_classes`);
* with the autotuner on (:func:`enable`), by timing every candidate on the
  first call of a class without an entry, on that call's own spectrum;
* otherwise from an occupancy model (most resident warps, then most CTAs).

Every call of one class in a process uses the same entry, so a stack gives the
same result alone and inside a batch.
"""

from __future__ import annotations

import ctypes
import json
from pathlib import Path
from typing import Iterable, List, Optional, Tuple

from . import _lib

TABLE_PATH = Path(__file__).resolve().parent / "tuning_table.json"
_PREC_NAME = {v: k for k, v in _lib.PREC.items()}
_MODE_NAME = {v: k for k, v in _lib.MODE.items()}


def enable(on: bool = True) -> None:
    """Switch the library's autotuner on (time candidates on a class's first call) or off."""
    _lib.load().fddm_b200_set_autotune(1 if on else 0)


def entries() -> List[dict]:
    """The library's tuning table as a list of dicts."""
    lib = _lib.load()
    out = []
    p, m, th, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    T, L = ctypes.c_uint64(), ctypes.c_uint64()
    for i in range(int(lib.fddm_b200_tuning_count())):
        _lib.check(lib.fddm_b200_tuning_entry(i, ctypes.byref(p), ctypes.byref(m), ctypes.byref(T), ctypes.byref(L),
                                              ctypes.byref(th), ctypes.byref(ns)))
        out.append({"precision": _PREC_NAME[p.value], "mode": _MODE_NAME[m.value], "frames": int(T.value),
                    "lags": int(L.value), "threads": int(th.value), "need_in_smem": int(ns.value)})
    return out


def set_entry(precision: str, mode: str, frames: int, lags: int, threads: int, need_in_smem: int) -> None:
    _lib.check(_lib.load().fddm_b200_tuning_set(_lib.PREC[precision], _lib.MODE[mode], int(frames), int(lags),
                                                 int(threads), int(need_in_smem)))


def lookup(precision: str, mode: str, frames: int, lags: int) -> Optional[Tuple[int, int]]:
    """(threads, need_in_smem) of a class, or None when the table has no entry."""
    lib = _lib.load()
    th, ns = ctypes.c_int(), ctypes.c_int()
    rc = lib.fddm_b200_tuning_get(_lib.PREC[precision], _lib.MODE[mode], int(frames), int(lags), ctypes.byref(th),
                                  ctypes.byref(ns))
    return (int(th.value), int(ns.value)) if rc == _lib.FDDM_OK else None


def load_table(path: Path = TABLE_PATH) -> int:
    """Load a saved table into the library; returns the number of entries."""
    if not Path(path).exists():
        return 0
    data = json.loads(Path(path).read_text())
    for e in data.get("entries", []):
        set_entry(e["precision"], e["mode"], e["frames"], e["lags"], e["threads"], e["need_in_smem"])
    return len(data.get("entries", []))


def save_table(path: Path = TABLE_PATH, device: str = "") -> None:
    rows = sorted(entries(), key=lambda e: (e["precision"], e["mode"], e["frames"], e["lags"]))
    Path(path).write_text(json.dumps({"device": device, "entries": rows}, indent=1) + "\n")


def tune_classes(classes: Iterable[Tuple], side: int = 192, gpu_id: int = 0) -> List[dict]:
    """Time every candidate launch shape for each (precision, mode, frames, nlags[, side]) class.

    Each class runs once on a synthetic stack of side x side frames (`side`
    unless the class names its own) with the autotuner on (a class already in
    the table is skipped); returns the table afterwards.
    """
    import numpy as np
    import torch

    from ._ddm_b200 import DdmPlan
    from ._fftopt import next_fast_len

    device = torch.device("cuda", gpu_id)
    enable(True)
    try:
        for cls in classes:
            precision, mode, T, nl = cls[:4]
            sd = cls[4] if len(cls) > 4 else side
            if lookup(precision, mode, T, nl) is not None:
                continue
            lags = np.unique(np.round(np.geomspace(1, T - 1, nl)).astype(int)) if nl < T - 1 else np.arange(1, T)
            if len(lags) != nl:  # geometric spacing collided: fill with the smallest unused lags
                extra = np.setdiff1d(np.arange(1, T), lags)[: nl - len(lags)]
                lags = np.sort(np.concatenate([lags, extra]))
            frames = torch.randint(0, 255, (T, sd, sd), dtype=torch.uint8, device=device)
            nt = next_fast_len(2 * T, "b200") if mode == "fft" else 0
            plan = DdmPlan(mode, T, sd, sd, 0, lags, sd, sd, nt, False, precision, device)
            out = torch.empty(plan.out_shape, dtype=torch.float64, device=device)
            plan.run(frames, None, out)
            torch.cuda.synchronize(device)
            del plan, out, frames
    finally:
        enable(False)
    return entries()


if __name__ == "__main__":  # pragma: no cover - run on a GB300 to refresh the committed table
    import argparse

    import numpy as np

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--out", default=str(TABLE_PATH))
    args = ap.parse_args()
    from . import synthetic

    # the benchmark workloads at their own frame sizes
    classes = [("ff", "fft", 4000, 200, 1024), ("ff", "fft", 512, 511, 512), ("ff", "fft", 64, 63, 128),
               ("ff", "fft", 20000, 200, 256), ("ff", "diff", 4000, 200, 1024), ("ff", "diff", 512, 511, 512),
               ("f64", "fft", 4000, 200, 1024), ("f32", "fft", 4000, 200, 1024)]
    # the uneven-stack batch: every length of the seeded 96-stack draw, all lags
    for sc in synthetic.config4_scenes(96, seed=0):
        classes.append(("ff", "fft", sc.length, sc.length - 1))
    classes = list(dict.fromkeys(classes))  # first occurrence of a class wins
    load_table(Path(args.out))
    tune_classes(classes)
    import torch

    save_table(Path(args.out), torch.cuda.get_device_name(0))
    print(f"{len(entries())} entries -> {args.out}")
