"""Image ingest: TIFF stacks into (optionally page-locked) host memory.

Interface of the reference's ``src/python/utils.py`` (``tiff2numpy`` ``:23-111``,
``images2numpy`` ``:114-163``, ``read_images`` ``:190-258``).  The reference
reads through tifffile / scikit-image / nd2reader; here grayscale TIFF files
(classic or BigTIFF, either byte order, strips, uncompressed, LZW or PackBits)
are decoded by the library's multithreaded reader (``fddm_b200_tiff_read``)
straight into the output array, which ``pinned=True`` places in page-locked
memory so that ``ddm`` uploads it asynchronously, overlapped with the spatial
FFTs.  Everything else (colour stacks with ``color_seq`` or ``input_order``,
tiled or otherwise compressed TIFFs, non-TIFF images, ND2) goes to the
reference's libraries when they are installed and raises otherwise.
"""

from __future__ import annotations

import ctypes
import os
import warnings
from concurrent.futures import ThreadPoolExecutor
from typing import List, Optional, Sequence, Union

import numpy as np

from . import _lib

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

_NP_DTYPE = {0: np.uint8, 1: np.int16, 2: np.uint16, 3: np.int32, 4: np.uint32, 5: np.int64, 6: np.uint64,
             7: np.float32, 8: np.float64}


def _threads() -> int:
    return max(1, min(16, os.cpu_count() or 1))


def _empty(shape, dtype, pinned: bool) -> np.ndarray:
    """Output array; page-locked (a view of a pinned torch tensor) when `pinned`."""
    if pinned and torch is not None and torch.cuda.is_available():
        t = torch.empty(int(np.prod(shape)) * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dtype).reshape(shape)  # the array keeps the tensor alive
    return np.empty(shape, dtype=dtype)


def tiff_info(src: str):
    """(pages, height, width, numpy dtype) of a TIFF file the native reader can decode."""
    lib = _lib.load()
    n, h, w, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_int()
    _lib.check(lib.fddm_b200_tiff_info(src.encode(), ctypes.byref(n), ctypes.byref(h), ctypes.byref(w),
                                       ctypes.byref(d)))
    return n.value, h.value, w.value, _NP_DTYPE[d.value]


def _read_pages(src: str, pages: np.ndarray, out: np.ndarray, nthreads: int) -> None:
    lib = _lib.load()
    idx = np.ascontiguousarray(pages, dtype=np.uint64)
    _lib.check(lib.fddm_b200_tiff_read(src.encode(), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                       len(idx), out.ctypes.data, nthreads))


def _fallback(what: str):
    try:
        import tifffile  # noqa: F401
    except ImportError as e:
        raise NotImplementedError(f"{what} needs tifffile, which is not installed") from e
    import tifffile

    return tifffile


def tiff2numpy(src: str, seq: Optional[Sequence[int]] = None, color_seq: Optional[Sequence[int]] = None,
               input_order: Optional[str] = None, *, pinned: bool = False) -> np.ndarray:
    """Read a (multipage) TIFF file as ``(T, Y, X)``; ``seq`` selects pages.

    Non-``.tif`` files are read with scikit-image's defaults, with a warning,
    as the reference does; ``color_seq`` and ``input_order`` (colour stacks)
    go to tifffile.
    """
    if not src.endswith(".tif"):
        warnings.warn("Non-tiff file, returning array opened with default settings only.")
        try:
            import skimage.io as io
        except ImportError as e:
            raise NotImplementedError("non-TIFF images need scikit-image, which is not installed") from e
        return io.imread(src)
    if color_seq is not None or input_order is not None:
        tifffile = _fallback("reading colour stacks (color_seq / input_order)")
        from_ref = tifffile.imread(src) if input_order is not None else tifffile.imread(src, key=color_seq)
        if input_order is not None:
            order = "CTYX"
            if len(input_order) != from_ref.ndim:
                raise RuntimeError(f"Given input dimensions '{input_order}' and loaded data shape "
                                   f"{from_ref.shape} mismatch:")
            if not all(d in order for d in input_order):
                raise RuntimeError(f"Unrecognized dimension in '{input_order}'. Only allowed values are '{order}'.")
            target = [d for d in order if d in input_order]
            from_ref = np.transpose(from_ref, axes=tuple(input_order.index(d) for d in target))
            if "C" in input_order:
                if color_seq is not None:
                    from_ref = from_ref[color_seq, ...]
                if seq is not None:
                    from_ref = from_ref[:, seq, ...]
            elif seq is not None:
                from_ref = from_ref[seq, ...]
            return from_ref
        return from_ref[:, seq, ...] if seq is not None else from_ref
    n, h, w, dtype = tiff_info(src)
    pages = np.arange(n, dtype=np.uint64) if seq is None else np.asarray(list(seq), dtype=np.int64)
    if seq is not None and (pages.size and (pages.min() < -n or pages.max() >= n)):
        raise IndexError(f"page index out of range for {n} pages")
    pages = np.where(pages < 0, pages + n, pages).astype(np.uint64) if seq is not None else pages
    out = _empty((len(pages), h, w), dtype, pinned)
    _read_pages(src, pages, out, _threads())
    if n == 1 and seq is None:
        return out[0]  # a single-page TIFF is one image (Y, X), as tifffile returns it
    return out


def images2numpy(fnames: Sequence[str], color_seq: Optional[Sequence[int]] = None, *,
                 pinned: bool = False) -> np.ndarray:
    """Read one image per file into ``(T, Y, X)`` (files read in parallel)."""
    if color_seq is not None or not all(str(f).endswith(".tif") for f in fnames):
        try:
            import skimage.io as io
        except ImportError as e:
            raise NotImplementedError("colour or non-TIFF images need scikit-image, which is not installed") from e
        first = io.imread(fnames[0])
        if first.ndim > 2:
            dim_y, dim_x, dim_col = first.shape
            cs = tuple(color_seq) if color_seq is not None else range(dim_col)
            seq = np.zeros((len(cs), len(fnames), dim_y, dim_x), dtype=first.dtype)
            for i, f in enumerate(fnames):
                tmp = io.imread(f)
                for j, c in enumerate(cs):
                    seq[j, i] = tmp[:, :, c]
            return seq
        seq = np.zeros((len(fnames), *first.shape), dtype=first.dtype)
        for i, f in enumerate(fnames):
            seq[i] = io.imread(f)
        return seq
    _, h, w, dtype = tiff_info(str(fnames[0]))
    out = _empty((len(fnames), h, w), dtype, pinned)
    zero = np.zeros(1, dtype=np.uint64)

    def one(i: int) -> None:
        f = str(fnames[i])
        _, hi, wi, di = tiff_info(f)
        if (hi, wi, di) != (h, w, dtype):
            raise RuntimeError(f"{f}: image shape or dtype differs from the first file")
        _read_pages(f, zero, out[i], 1)

    with ThreadPoolExecutor(max_workers=_threads()) as ex:
        list(ex.map(one, range(len(fnames))))
    return out


def read_images(src: Union[str, List[str]], seq: Optional[Sequence[int]] = None,
                color_seq: Optional[Sequence[int]] = None, input_order: Optional[str] = None, *,
                pinned: bool = False) -> np.ndarray:
    """Read a single image file or a list of image files (``src/python/utils.py:190-258``).

    ``pinned=True`` returns the frames in page-locked memory (TIFF path), which
    ``ddm`` uploads asynchronously, overlapped with its spatial FFTs.
    """
    if isinstance(src, list):
        return images2numpy(src, color_seq=color_seq, pinned=pinned)
    if isinstance(src, str):
        if src.endswith(".nd2"):
            try:
                from nd2reader import ND2Reader
            except ImportError as e:
                raise NotImplementedError("ND2 files need nd2reader, which is not installed") from e
            mov = ND2Reader(src)
            length, dim_y, dim_x = mov.shape
            selected = list(seq) if seq is not None else range(length)
            imgs = np.zeros((len(selected), dim_y, dim_x), dtype=mov[0].dtype)
            for i, idx in enumerate(selected):
                imgs[i] = mov.get_frame(idx).data
            return imgs
        return tiff2numpy(src, seq=seq, color_seq=color_seq, input_order=input_order, pinned=pinned)
    raise RuntimeError(f"Failed to open {src}.")
