"""Minimal image I/O for films and golden images (numpy + zlib only).

PNG decoding covers what the reference's golden images use: bit depths 1-16,
grey / grey+alpha / RGB / RGBA / palette colour types, non-interlaced. PPM (P6)
is what the reference's CImg writer produces for ``--output=*.ppm``
(film.cc:42 calls CImg::save, which writes binary PPM natively).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    pos = 0
    for y in range(height):
        ftype = raw[pos]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=pos + 1).astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype in (1, 3, 4):
            cur = line.copy()
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                if ftype == 1:
                    cur[x] = (cur[x] + a) & 0xFF
                elif ftype == 3:
                    cur[x] = (cur[x] + ((a + b) >> 1)) & 0xFF
                else:
                    c = prev[x - bpp] if x >= bpp else 0
                    cur[x] = (cur[x] + _paeth(a, b, c)) & 0xFF
        else:
            raise ValueError(f"bad PNG filter type {ftype}")
        out[y] = cur
        prev = cur
    return out


def read_png(path: str) -> np.ndarray:
    """Return an (H, W, 3) uint8 RGB array (16-bit samples keep the high byte)."""
    data = open(path, "rb").read()
    if data[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG")
    pos = 8
    idat = b""
    palette = None
    width = height = depth = ctype = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            if interlace:
                raise ValueError("interlaced PNG unsupported")
        elif kind == b"PLTE":
            palette = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits_pp = channels * depth
    stride = (width * bits_pp + 7) // 8
    bpp = max(1, bits_pp // 8)
    rows = _unfilter(zlib.decompress(idat), height, stride, bpp)
    if depth < 8:
        bits = np.unpackbits(rows, axis=1)[:, : width * depth].reshape(height, width, depth)
        weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
        samples = (bits * weights).sum(axis=2).astype(np.uint16)[..., None]
    elif depth == 8:
        samples = rows.reshape(height, width, channels).astype(np.uint16)
    else:
        samples = rows.reshape(height, width, channels, 2)[..., 0].astype(np.uint16)
    if ctype == 3:
        return palette[samples[..., 0]]
    if ctype in (0, 4):
        g = samples[..., 0]
        if depth < 8:
            g = g * 255 // ((1 << depth) - 1)
        return np.repeat(g[..., None], 3, axis=2).astype(np.uint8)
    return samples[..., :3].astype(np.uint8)


def read_ppm(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    tokens = []
    pos = 0
    while len(tokens) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            while data[pos:pos + 1] not in (b"\n", b""):
                pos += 1
            continue
        start = pos
        while not data[pos:pos + 1].isspace():
            pos += 1
        tokens.append(data[start:pos])
    if tokens[0] != b"P6":
        raise ValueError(f"{path}: only binary PPM (P6) supported")
    w, h, maxval = int(tokens[1]), int(tokens[2]), int(tokens[3])
    pos += 1
    if maxval > 255:
        arr = np.frombuffer(data, dtype=">u2", count=w * h * 3, offset=pos).reshape(h, w, 3)
        return (arr >> 8).astype(np.uint8)
    return np.frombuffer(data, dtype=np.uint8, count=w * h * 3, offset=pos).reshape(h, w, 3).copy()


def read_image(path: str) -> np.ndarray:
    return read_png(path) if path.lower().endswith(".png") else read_ppm(path)


def write_png(path: str, rgb: np.ndarray) -> None:
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(kind: bytes, body: bytes) -> bytes:
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    png = _PNG_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    open(path, "wb").write(png)
