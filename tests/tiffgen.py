"""Minimal TIFF writer for the ingest tests (test infrastructure only).

Follows the TIFF 6.0 specification (baseline IFD layout, PackBits,
LZW with the code-width switch of the libtiff family, horizontal
differencing predictor) and the BigTIFF extension (magic 43, 8-byte offsets).
"""

from __future__ import annotations

import struct
from typing import List, Sequence

import numpy as np


def packbits(data: bytes) -> bytes:
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j > i:  # run of data[i], length j - i + 1 >= 2
            out += bytes([(257 - (j - i + 1)) & 0xFF, data[i]])
            i = j + 1
            continue
        k = i
        while k < n and k - i < 128 and not (k + 1 < n and data[k + 1] == data[k]):
            k += 1
        k = max(k, i + 1)
        out += bytes([k - i - 1]) + data[i:k]
        i = k
    return bytes(out)


def lzw(data: bytes) -> bytes:
    bits: List[int] = []
    width = 9

    def put(code: int) -> None:
        for b in range(width - 1, -1, -1):
            bits.append((code >> b) & 1)

    table = {bytes([i]): i for i in range(256)}
    nxt = 258
    put(256)
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        put(table[w])
        table[wc] = nxt
        nxt += 1
        if nxt == 4094:
            put(256)
            table = {bytes([i]): i for i in range(256)}
            nxt = 258
            width = 9
        elif nxt > (1 << width) - 1 and width < 12:
            width += 1
        w = bytes([c])
    if w:
        put(table[w])
    put(257)
    while len(bits) % 8:
        bits.append(0)
    return bytes(int("".join(map(str, bits[i:i + 8])), 2) for i in range(0, len(bits), 8))


def write_tiff(path, pages: Sequence[np.ndarray], *, byteorder: str = "<", bigtiff: bool = False,
               rows_per_strip: int = 0, compression: str = "none", predictor: bool = False) -> None:
    """Write 2-D arrays as the pages of one grayscale TIFF file."""
    bo = byteorder
    pages = [np.asarray(p) for p in pages]
    dt = pages[0].dtype
    fmt = {"u": 1, "i": 2, "f": 3}[dt.kind]
    comp = {"none": 1, "lzw": 5, "packbits": 32773}[compression]
    buf = bytearray()
    buf += (b"II" if bo == "<" else b"MM")
    if bigtiff:
        buf += struct.pack(bo + "HHHQ", 43, 8, 0, 0)
    else:
        buf += struct.pack(bo + "HI", 42, 0)
    first_ptr = 8 if bigtiff else 4  # where the first IFD offset goes
    prev_ptr = first_ptr
    for img in pages:
        h, w = img.shape
        rps = rows_per_strip or h
        raw = img.astype(img.dtype.newbyteorder(bo))
        offsets, counts = [], []
        for r0 in range(0, h, rps):
            block = raw[r0:r0 + rps].copy()
            if predictor:
                nat = img[r0:r0 + rps].copy()
                diff = nat.copy()
                diff[:, 1:] = nat[:, 1:] - nat[:, :-1]  # wraps in the integer type
                block = diff.astype(img.dtype.newbyteorder(bo))
            data = block.tobytes()
            if comp == 5:
                data = lzw(data)
            elif comp == 32773:
                data = packbits(data)
            offsets.append(len(buf))
            counts.append(len(data))
            buf += data
            if len(buf) % 2:
                buf += b"\0"
        ifd_off = len(buf)
        struct.pack_into(bo + ("Q" if bigtiff else "I"), buf, prev_ptr, ifd_off)
        nstrips = len(offsets)
        ltype = 16 if bigtiff else 4
        entries = [(256, 4, [w]), (257, 4, [h]), (258, 3, [img.dtype.itemsize * 8]), (259, 3, [comp]),
                   (262, 3, [1]), (273, ltype, offsets), (277, 3, [1]), (278, 4, [rps]), (279, ltype, counts),
                   (339, 3, [fmt])]
        if predictor:
            entries.append((317, 3, [2]))
        entries.sort()
        esz, csz, inl = (20, 8, 8) if bigtiff else (12, 2, 4)
        tsz = {3: 2, 4: 4, 16: 8}
        tfmt = {3: "H", 4: "I", 16: "Q"}
        ifd_len = csz + len(entries) * esz + (8 if bigtiff else 4)
        extra_off = ifd_off + ifd_len
        extra = bytearray()
        ifd = bytearray(struct.pack(bo + ("Q" if bigtiff else "H"), len(entries)))
        for tag, typ, vals in entries:
            payload = b"".join(struct.pack(bo + tfmt[typ], v) for v in vals)
            head = struct.pack(bo + ("HHQ" if bigtiff else "HHI"), tag, typ, len(vals))
            if len(payload) <= inl:
                ifd += head + payload + bytes(inl - len(payload))
            else:
                ifd += head + struct.pack(bo + ("Q" if bigtiff else "I"), extra_off + len(extra))
                extra += payload
        prev_ptr = ifd_off + len(ifd)
        ifd += bytes(8 if bigtiff else 4)  # next IFD: patched by the next page
        buf += ifd + extra
        del nstrips, tsz
    with open(path, "wb") as f:
        f.write(bytes(buf))
