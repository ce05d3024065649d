"""A small PNG decoder for the test harness (the reference's regression
images are PNG files and libpng is not available).  It follows the PNG
specification (ISO/IEC 15948): chunk layout, zlib stream, the five row
filters, Adam7 interlacing, bit depths 1-16 for every colour type, and the
ancillary chunks that change how ImageWorsener reads a file (PLTE, tRNS,
sBIT, gAMA, sRGB, bKGD, pHYs).

Test infrastructure only: nothing in the library uses it.
"""
from __future__ import annotations

import struct
import zlib
from dataclasses import dataclass, field

import numpy as np

SIGNATURE = b"\x89PNG\r\n\x1a\n"
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}   # colour type -> samples per pixel
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


@dataclass
class PNG:
    width: int
    height: int
    bit_depth: int
    color_type: int
    interlaced: bool
    samples: np.ndarray                     # (h, w, channels) uint16, as stored (palette: indices)
    palette: np.ndarray | None = None       # (n, 3) uint8
    trns: bytes | None = None               # raw tRNS payload
    sbit: tuple[int, ...] | None = None
    gamma: float | None = None              # gAMA / 100000
    srgb_intent: int | None = None
    bkgd: tuple[int, ...] | None = None
    phys: tuple[int, int, int] | None = None
    chunks: list[str] = field(default_factory=list)

    @property
    def channels(self) -> int:
        return CHANNELS[self.color_type]


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(data: bytes, pos: int, rows: int, rowbytes: int, bpp: int) -> tuple[list[bytearray], int]:
    """Undo the per-row filters of one (sub)image; bpp = bytes per complete
    pixel, at least 1."""
    out: list[bytearray] = []
    prev = bytearray(rowbytes)
    for _ in range(rows):
        ftype = data[pos]
        cur = bytearray(data[pos + 1:pos + 1 + rowbytes])
        pos += 1 + rowbytes
        if ftype == 1:
            for i in range(bpp, rowbytes):
                cur[i] = (cur[i] + cur[i - bpp]) & 255
        elif ftype == 2:
            for i in range(rowbytes):
                cur[i] = (cur[i] + prev[i]) & 255
        elif ftype == 3:
            for i in range(rowbytes):
                left = cur[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + ((left + prev[i]) >> 1)) & 255
        elif ftype == 4:
            for i in range(rowbytes):
                left = cur[i - bpp] if i >= bpp else 0
                up_left = prev[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + _paeth(left, prev[i], up_left)) & 255
        elif ftype != 0:
            raise ValueError("bad PNG filter type %d" % ftype)
        out.append(cur)
        prev = cur
    return out, pos


def _row_samples(row: bytes, width: int, channels: int, depth: int) -> np.ndarray:
    n = width * channels
    if depth == 16:
        return np.frombuffer(bytes(row), dtype=">u2")[:n].astype(np.uint16)
    if depth == 8:
        return np.frombuffer(bytes(row), dtype=np.uint8)[:n].astype(np.uint16)
    bits = np.unpackbits(np.frombuffer(bytes(row), dtype=np.uint8))
    vals = bits.reshape(-1, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
    return (vals.astype(np.uint16) * weights).sum(axis=1).astype(np.uint16)[:n]


def read_png(path: str) -> PNG:
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != SIGNATURE:
        raise ValueError("not a PNG file")
    pos, idat, info = 8, [], {}
    names = []
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8].decode("latin-1")
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        names.append(ctype)
        if ctype == "IHDR":
            w, h, depth, color, _, _, interlace = struct.unpack(">IIBBBBB", body)
            info.update(width=w, height=h, bit_depth=depth, color_type=color, interlaced=interlace == 1)
        elif ctype == "PLTE":
            info["palette"] = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3).copy()
        elif ctype == "tRNS":
            info["trns"] = bytes(body)
        elif ctype == "sBIT":
            info["sbit"] = tuple(body)
        elif ctype == "gAMA":
            info["gamma"] = struct.unpack(">I", body)[0] / 100000.0
        elif ctype == "sRGB":
            info["srgb_intent"] = body[0]
        elif ctype == "bKGD":
            info["bkgd"] = tuple(body) if len(body) == 1 else struct.unpack(">%dH" % (len(body) // 2), body)
        elif ctype == "pHYs":
            info["phys"] = struct.unpack(">IIB", body)
        elif ctype == "IDAT":
            idat.append(body)
        elif ctype == "IEND":
            break
    raw = zlib.decompress(b"".join(idat))
    w, h, depth, color = info["width"], info["height"], info["bit_depth"], info["color_type"]
    ch = CHANNELS[color]
    bpp = max(1, ch * depth // 8)
    samples = np.zeros((h, w, ch), dtype=np.uint16)
    if not info["interlaced"]:
        rows, _ = _unfilter(raw, 0, h, (w * ch * depth + 7) // 8, bpp)
        for y, row in enumerate(rows):
            samples[y] = _row_samples(row, w, ch, depth).reshape(w, ch)
    else:
        p = 0
        for x0, y0, dx, dy in ADAM7:
            sw, sh = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
            if sw <= 0 or sh <= 0:
                continue
            rows, p = _unfilter(raw, p, sh, (sw * ch * depth + 7) // 8, bpp)
            for j, row in enumerate(rows):
                samples[y0 + j * dy, x0::dx][:sw] = _row_samples(row, sw, ch, depth).reshape(sw, ch)
    return PNG(samples=samples, chunks=names, **info)
