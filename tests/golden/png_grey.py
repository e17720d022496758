"""Grey images from 8-bit PNG files with the standard library only (zlib):
the reader the stereo fixtures use, since neither OpenCV nor PIL is present.

Supports the PNG colour types the reference example's pair uses (grey, RGB,
RGBA; 8 bits, no interlace) and all five row filters of the PNG
specification (ISO/IEC 15948, section 9).  Colour pixels become grey by the
fixed integer luma map (299 R + 587 G + 114 B + 500) / 1000.  Test
infrastructure only."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _unfilter(raw: bytes, h: int, stride: int, ch: int) -> np.ndarray:
    out = np.zeros((h, stride), np.int64)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)], np.uint8).astype(np.int64)
        if f == 0:
            cur = line.copy()
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, np.int64)
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) // 2
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    return out


def grey(path: str) -> np.ndarray:
    """(H, W) uint8 grey image of an 8-bit grey / RGB / RGBA PNG."""
    data = open(path, "rb").read()
    w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", data[16:29])
    if depth != 8 or interlace != 0 or ctype not in (0, 2, 6):
        raise ValueError(f"{path}: only 8-bit, non-interlaced grey / RGB / RGBA PNGs are read")
    chunks, pos = b"", 8
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        if data[pos + 4:pos + 8] == b"IDAT":
            chunks += data[pos + 8:pos + 8 + n]
        pos += 12 + n
    ch = {0: 1, 2: 3, 6: 4}[ctype]
    px = _unfilter(zlib.decompress(chunks), h, w * ch, ch).reshape(h, w, ch)
    if ch == 1:
        return px[:, :, 0].astype(np.uint8)
    r, g, b = px[:, :, 0], px[:, :, 1], px[:, :, 2]
    return ((r * 299 + g * 587 + b * 114 + 500) // 1000).astype(np.uint8)


def stereo_costs_u8(left: np.ndarray, right: np.ndarray, L: int, cap: int) -> np.ndarray:
    """The reference example's integer cost volume (examples/stereo/stereo.cc:28-34),
    label-planar (L, H, W) int32: min(|left(x) - right(x-k)|, cap) for
    x >= L-1, zero in the columns x < L-1."""
    H, W = left.shape
    a, b = left.astype(np.int32), right.astype(np.int32)
    D = np.zeros((L, H, W), np.int32)
    for k in range(L):
        D[k, :, L - 1:] = np.minimum(np.abs(a[:, L - 1:] - b[:, L - 1 - k:W - k]), cap)
    return D
