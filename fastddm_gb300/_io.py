"""Binary files of the image structure function (``.sf.ddm``), its azimuthal
average (``.aa.ddm``) and the intermediate scattering function (``.isf.ddm``),
byte-compatible with the reference's writers and readers.

Formats (reference ``src/python/_io_common.py:16-17`` for the version (0, 3)
and the 64-byte header, ``imagestructurefunction.py:409-627, 629-884`` for
``.sf.ddm``, ``azimuthalaverage.py:567-753, 755-976`` for ``.aa.ddm``,
``intermediatescatteringfunction.py:213-623`` for ``.isf.ddm``, the ``.aa.ddm``
layout with another identifier): a header with the byte order ("LL"/"BB"),
the file identifier (73, 22 or 43), the
version, the dtype character and the sizes, then the arrays in C order, then
the byte offsets of every array, written in reverse so that a reader starts
from the end of the file.

The ``.sf.ddm`` writer is native (``fddm_b200_sf_write``): from host memory it
is one sequential write; from device memory it streams the structure function
through pinned staging buffers, overlapping each device-to-host copy with the
write of the previous chunk (``ddm_save`` computes and writes a stack without
ever holding the result in host memory).  ``.aa.ddm`` and ``.isf.ddm`` files
are small and are written here with ``struct``.
"""

from __future__ import annotations

import os
import struct
import sys
from pathlib import Path
from typing import Any, Optional, Sequence, Tuple, Union

import numpy as np

from . import _lib
from .azimuthalaverage import AzimuthalAverage
from .imagestructurefunction import ImageStructureFunction, _reconstruct_full_spectrum

VERSION = (0, 3)
HEAD_BYTE_LEN = 64
SF_ID = 73
AA_ID = 22
ISF_ID = 43

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _with_suffix(fname: str, suffix: str) -> str:
    """The reference's naming rule (``imagestructurefunction.py:287-292``): add the suffix if missing."""
    d, name = os.path.split(fname)
    name = name if name.endswith(suffix) else f"{name}{suffix}"
    path = os.path.join(d, name)
    Path(os.path.dirname(path) or ".").mkdir(parents=True, exist_ok=True)
    return path


# ---------------------------------------------------------------------------
# .sf.ddm
# ---------------------------------------------------------------------------
def sf_write(path: str, data, kx: np.ndarray, ky: np.ndarray, tau: np.ndarray, width: int, height: int,
             pixel_size: float = 1.0, delta_t: float = 1.0) -> None:
    """Write ``data`` (``(len(tau) + 2, ny, nx//2 + 1)`` float64, numpy or a CUDA
    tensor) with its axes to ``path`` in the ``.sf.ddm`` format."""
    on_device = torch is not None and isinstance(data, torch.Tensor) and data.is_cuda
    if on_device:
        if data.dtype != torch.float64 or not data.is_contiguous():
            raise ValueError("device data must be a contiguous float64 tensor")
        shape = tuple(data.shape)
        ptr = data.data_ptr()
        stream = torch.cuda.current_stream(data.device)
        sptr = stream.cuda_stream
        keep = data
    else:
        keep = np.ascontiguousarray(data, dtype=np.float64)
        shape = keep.shape
        ptr = keep.ctypes.data
        sptr = None
    if len(shape) != 3:
        raise ValueError("data must have shape (lags + extra, ny, nx//2 + 1)")
    kx = np.ascontiguousarray(kx, dtype=np.float64)
    ky = np.ascontiguousarray(ky, dtype=np.float64)
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    length = len(tau)
    extra = shape[0] - length
    if extra < 0 or len(kx) != shape[2] or len(ky) != shape[1]:
        raise ValueError("axis lengths do not match the data shape")
    lib = _lib.load()
    if on_device:
        with torch.cuda.device(keep.device):
            rc = lib.fddm_b200_sf_write(str(path).encode(), ptr, 1, length, shape[1], shape[2], extra, int(width),
                                        int(height), kx.ctypes.data, ky.ctypes.data, tau.ctypes.data,
                                        float(pixel_size), float(delta_t), sptr)
    else:
        rc = lib.fddm_b200_sf_write(str(path).encode(), ptr, 0, length, shape[1], shape[2], extra, int(width),
                                    int(height), kx.ctypes.data, ky.ctypes.data, tau.ctypes.data,
                                    float(pixel_size), float(delta_t), sptr)
    _lib.check(rc)


def save_sf(obj: ImageStructureFunction, fname: str = "analysis_blob", from_device: bool = False) -> str:
    """``ImageStructureFunction.save``: write ``obj`` to ``fname`` (``.sf.ddm`` appended if missing).

    ``from_device`` streams the object's device copy of ``_data`` instead of
    its host array.  Returns the path written.
    """
    path = _with_suffix(fname, ".sf.ddm")
    data = obj._device_data if (from_device and obj._device_data is not None) else obj._data
    sf_write(path, data, obj.kx, obj.ky, obj.tau, obj.width, obj.height, obj.pixel_size, obj.delta_t)
    return path


def ddm_save(img_seq, lags, fname: str, *, mode: str = "fft", window: Optional[np.ndarray] = None,
             pixel_size: float = 1.0, delta_t: float = 1.0, **kwargs) -> str:
    """Compute the image structure function on the GB300 and write it straight
    to ``fname`` (``.sf.ddm``) from device memory; the result is never copied
    to host memory as a whole.  Same arguments and checks as ``ddm``; returns
    the path written."""
    from ._ddm import _prepare
    from ._ddm_b200 import ddm_device

    lags, window, nx, ny, nt, kx, ky = _prepare(img_seq, lags, "b200", mode, window)
    out = ddm_device(img_seq, lags, nx, ny, nt, window, mode=mode, **kwargs)
    path = _with_suffix(fname, ".sf.ddm")
    sf_write(path, out, kx, ky, lags.astype(np.float64), nx, ny, pixel_size, delta_t)
    return path


class _Parser:
    """Header and offset parsing shared by both file kinds (``_io_common.py:178-353``)."""

    supported_file_versions = {(0, 1): False, (0, 2): False, (0, 3): True}

    def __init__(self, fh, file_id: int, kind: str):
        self._fh = fh
        fh.seek(0)
        flag = fh.read(2).decode("utf-8")
        if flag == "LL":
            self.byteorder = "<"
        elif flag == "BB":
            self.byteorder = ">"
        else:
            raise RuntimeError(f"Byteorder {flag} not recognized. Input file might be corrupted.")
        fh.seek(6)
        self.dtype = fh.read(1).decode("utf-8")
        ident = self.read_value(2, "H")
        if ident != file_id:
            raise RuntimeError(f"File identifier {ident} not compatible with {kind} file ({file_id})."
                               " Input file might be wrong or corrupted.")
        self.version = (self.read_value(4, "B"), self.read_value(5, "B"))
        self.supported = bool(self.supported_file_versions.get(self.version))

    def read_value(self, offset: int, fmt: str, whence: int = 0) -> Any:
        self._fh.seek(offset, whence)
        return struct.unpack(self.byteorder + fmt, self._fh.read(struct.calcsize(fmt)))[0]

    def read_array(self, offset: int, shape) -> np.ndarray:
        count = int(np.prod(shape))
        self._fh.seek(0)
        return np.fromfile(self._fh, np.dtype(self.byteorder + self.dtype), count, offset=offset).reshape(shape)

    def offsets_from_end(self, n: int):
        q = struct.calcsize("Q")
        vals = [self.read_value(-q, "Q", 2)]
        for _ in range(n - 1):
            vals.append(self.read_value(-2 * q, "Q", 1))
        return vals


class SFReader:
    """Reader of ``.sf.ddm`` files (interface of ``imagestructurefunction.py:629-832``)."""

    def __init__(self, file: str):
        self._fh = open(file, "rb")
        self._parser = _Parser(self._fh, SF_ID, "image structure function")
        p = self._parser
        m = {"Nt": p.read_value(7, "Q")}
        for key in ("Ny", "Nx", "Nextra", "width", "height"):
            m[key] = p.read_value(0, "Q", 1)
        (m["data_offset"], m["kx_offset"], m["ky_offset"], m["tau_offset"], ps_off, dt_off,
         m["extra_offset"]) = p.offsets_from_end(7)
        m["pixel_size"] = p.read_value(ps_off, p.dtype)
        m["delta_t"] = p.read_value(dt_off, p.dtype)
        self._metadata = m

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def close(self) -> None:
        if self._fh:
            self._fh.close()

    def load(self) -> ImageStructureFunction:
        if not self._parser.supported:
            raise IOError(f"File version {self._parser.version} not supported.")
        m = self._metadata
        data = self._parser.read_array(m["data_offset"], (m["Nt"] + m["Nextra"], m["Ny"], m["Nx"]))
        return ImageStructureFunction(data, self.get_kx(False), self.get_ky(False), m["width"], m["height"],
                                      self.get_tau(), m["pixel_size"], m["delta_t"])

    def get_kx(self, full: bool = True) -> np.ndarray:
        m = self._metadata
        kx = self._parser.read_array(m["kx_offset"], m["Nx"])
        if not full:
            return kx
        out = np.zeros_like(kx, shape=m["width"])
        out[: m["Nx"]] = kx
        out[m["Nx"]:] = -np.flip(kx[1:-1]) if m["width"] % 2 == 0 else -np.flip(kx[1:])
        return np.fft.fftshift(out)

    def get_ky(self, full: bool = True) -> np.ndarray:
        m = self._metadata
        return self._parser.read_array(m["ky_offset"], m["Ny"])

    def get_tau(self) -> np.ndarray:
        m = self._metadata
        return self._parser.read_array(m["tau_offset"], m["Nt"])

    def _plane(self, offset: int, full: bool) -> np.ndarray:
        m = self._metadata
        plane = self._parser.read_array(offset, (m["Ny"], m["Nx"]))
        return _reconstruct_full_spectrum(plane, (m["height"], m["width"])) if full else plane

    def get_frame(self, index: int, full: bool = True) -> np.ndarray:
        m = self._metadata
        if index < 0 or index >= m["Nt"]:
            raise IndexError(f"Index out of range. Choose an index between 0 and {m['Nt'] - 1}.")
        es = struct.calcsize(self._parser.dtype)
        return self._plane(m["data_offset"] + index * m["Nx"] * m["Ny"] * es, full)

    def get_power_spec(self, full: bool = True) -> np.ndarray:
        return self._plane(self._metadata["extra_offset"], full)

    def get_var(self, full: bool = True) -> np.ndarray:
        m = self._metadata
        es = struct.calcsize(self._parser.dtype)
        return self._plane(m["extra_offset"] + m["Nx"] * m["Ny"] * es, full)


# ---------------------------------------------------------------------------
# .aa.ddm
# ---------------------------------------------------------------------------
def save_aa(obj: AzimuthalAverage, fname: str = "analysis_blob") -> str:
    """``AzimuthalAverage.save``: write ``obj`` to ``fname`` (``.aa.ddm`` appended if missing)."""
    return _save_binned(obj, _with_suffix(fname, ".aa.ddm"), AA_ID)


def save_isf(obj, fname: str = "analysis_blob") -> str:
    """``IntermediateScatteringFunction.save``: the ``.aa.ddm`` layout with file identifier 43
    (``intermediatescatteringfunction.py:213-400``)."""
    return _save_binned(obj, _with_suffix(fname, ".isf.ddm"), ISF_ID)


def _save_binned(obj, path: str, file_id: int) -> str:
    """Binned (k, tau) data with optional errors, k, tau and bin edges."""
    data = np.ascontiguousarray(obj._data)
    if data.dtype == np.float64:
        fmt = "d"
    elif data.dtype == np.float32:
        fmt = "f"
    else:
        raise NotImplementedError(f"Numpy dtype to binary format converter not implemented for type {data.dtype}.")
    es = struct.calcsize(fmt)
    Nt = len(obj.tau)
    Nk, dim_t = data.shape
    Nextra = dim_t - Nt
    is_err = obj._err is not None
    head = ("LL" if sys.byteorder == "little" else "BB").encode() + struct.pack("H", file_id)
    head += struct.pack("BB", *VERSION) + fmt.encode() + struct.pack("QQQ", Nk, Nt, Nextra)
    head += struct.pack("B", 1 if is_err else 0)
    head += bytes(HEAD_BYTE_LEN - len(head))
    data_off = HEAD_BYTE_LEN
    err_off = data_off + Nk * (Nt + Nextra) * es
    k_off = err_off + (Nk * (Nt + Nextra) * es if is_err else 0)
    tau_off = k_off + Nk * es
    edges_off = tau_off + Nt * es
    with open(path, "wb") as fh:
        fh.write(head)
        data.tofile(fh)
        if is_err:
            np.ascontiguousarray(obj._err).tofile(fh)
        for a in (obj.k, obj.tau, obj.bin_edges):
            np.ascontiguousarray(a).tofile(fh)
        fh.write(struct.pack("QQQQQ", edges_off, tau_off, k_off, err_off, data_off))
    return path


class AAReader:
    """Reader of ``.aa.ddm`` files (interface of ``azimuthalaverage.py:755-911``)."""

    _id, _kind = AA_ID, "azimuthal average"

    def _make(self, data, err, k, tau, bin_edges):
        return AzimuthalAverage(data, err, k, tau, bin_edges)

    def __init__(self, file: str):
        self._fh = open(file, "rb")
        self._parser = p = _Parser(self._fh, self._id, self._kind)
        m = {"Nk": p.read_value(7, "Q")}
        m["Nt"] = p.read_value(0, "Q", 1)
        m["Nextra"] = p.read_value(0, "Q", 1)
        newer = p.version > (0, 1)
        m["is_err"] = bool(p.read_value(0, "B", 1)) if newer else False
        if newer:
            (m["data_offset"], m["err_offset"], m["k_offset"], m["tau_offset"],
             m["bin_edges_offset"]) = p.offsets_from_end(5)
        else:
            m["data_offset"], m["k_offset"], m["tau_offset"], m["bin_edges_offset"] = p.offsets_from_end(4)
            m["err_offset"] = 0
        self._metadata = m

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def close(self) -> None:
        if self._fh:
            self._fh.close()

    def load(self) -> AzimuthalAverage:
        if not self._parser.supported:
            raise IOError(f"File version {self._parser.version} not supported.")
        m = self._metadata
        shape = (m["Nk"], m["Nt"] + m["Nextra"])
        err = self._parser.read_array(m["err_offset"], shape) if m["is_err"] else None
        return self._make(self._parser.read_array(m["data_offset"], shape), err, self.get_k(), self.get_tau(),
                          self.get_bin_edges())

    def get_k(self) -> np.ndarray:
        return self._parser.read_array(self._metadata["k_offset"], self._metadata["Nk"])

    def get_tau(self) -> np.ndarray:
        return self._parser.read_array(self._metadata["tau_offset"], self._metadata["Nt"])

    def get_bin_edges(self) -> np.ndarray:
        return self._parser.read_array(self._metadata["bin_edges_offset"], self._metadata["Nk"])

    def _k_row(self, offset_key: str, k_index: int) -> np.ndarray:
        m = self._metadata
        if k_index < 0 or k_index >= m["Nk"]:
            raise IndexError(f"Index out of range. Choose an index between 0 and {m['Nk'] - 1}.")
        es = struct.calcsize(self._parser.dtype)
        return self._parser.read_array(m[offset_key] + k_index * (m["Nt"] + m["Nextra"]) * es, m["Nt"])

    def get_k_slice(self, k_index: int) -> np.ndarray:
        return self._k_row("data_offset", k_index)

    def get_k_slice_err(self, k_index: int) -> Optional[np.ndarray]:
        row = self._k_row("err_offset", k_index)
        return row if self._metadata["is_err"] else None


class ISFReader(AAReader):
    """Reader of ``.isf.ddm`` files (interface of ``intermediatescatteringfunction.py:402-559``)."""

    _id, _kind = ISF_ID, "intermediate scattering function"

    def _make(self, data, err, k, tau, bin_edges):
        from .intermediatescatteringfunction import IntermediateScatteringFunction

        return IntermediateScatteringFunction(data, err, k, tau, bin_edges)


def load(fname: str):
    """Read a ``.sf.ddm``, ``.aa.ddm`` or ``.isf.ddm`` file (``src/python/_io.py:14-36``)."""
    if fname.endswith(".sf.ddm"):
        with SFReader(fname) as f:
            return f.load()
    if fname.endswith(".aa.ddm"):
        with AAReader(fname) as f:
            return f.load()
    if fname.endswith(".isf.ddm"):
        with ISFReader(fname) as f:
            return f.load()
    raise RuntimeError("File extension not recognized.")
