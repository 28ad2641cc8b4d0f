"""A PNG encoder for the decoder tests (Python's zlib for DEFLATE): every
colour type and bit depth, per-row filter types, Adam7 interlacing, tRNS,
split IDAT chunks, and the expected RGBA8 of the decoder's conversion rules."""
from __future__ import annotations

import struct
import zlib

import numpy as np

CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """One scanline of samples (already flattened) at `depth` bits."""
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    if depth == 16:
        return samples.astype(">u2").tobytes()
    per = 8 // depth
    n = samples.size
    out = bytearray((n * depth + 7) // 8)
    for i, v in enumerate(samples.tolist()):
        out[i // per] |= int(v) << (8 - depth * (i % per + 1))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter(raw: bytes, prev: bytes, ft: int, bpp: int) -> bytes:
    out = bytearray(len(raw))
    for i in range(len(raw)):
        a = raw[i - bpp] if i >= bpp else 0
        b = prev[i] if prev else 0
        c = prev[i - bpp] if (prev and i >= bpp) else 0
        pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
        out[i] = (raw[i] - pred) & 0xFF
    return bytes(out)


def encode(samples: np.ndarray, ctype: int, depth: int, rng, interlace: bool = False, palette=None, trns=None,
           level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY, idat_split: int = 0) -> bytes:
    """samples: (H, W, channels) integer samples at `depth` bits."""
    h, w, ch = samples.shape
    assert ch == CHANNELS[ctype]
    bits_pp = depth * ch
    bpp = max(1, bits_pp // 8)
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    stream = bytearray()
    for ox, oy, sx, sy in passes:
        sub = samples[oy::sy, ox::sx]
        if sub.size == 0:
            continue
        prev = b""
        for row in sub:
            raw = _pack_row(row.reshape(-1), depth)
            ft = int(rng.integers(0, 5))
            stream += bytes([ft]) + _filter(raw, prev, ft, bpp)
            prev = raw
    comp = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
    data = comp.compress(bytes(stream)) + comp.flush()
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if palette is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += _chunk(b"tRNS", trns)
    if idat_split:
        for k in range(0, len(data), idat_split):
            png += _chunk(b"IDAT", data[k:k + idat_split])
    else:
        png += _chunk(b"IDAT", data)
    png += _chunk(b"tEXt", b"Comment\x00an ancillary chunk the decoder skips")
    return png + _chunk(b"IEND", b"")


def expected_rgba(samples: np.ndarray, ctype: int, depth: int, palette=None, trns=None) -> np.ndarray:
    """The decoder's RGBA8: 16-bit samples keep their high byte, 1/2/4-bit
    gray is scaled by 255 / (2^d - 1), palette entries and tRNS alpha."""
    s = samples.astype(np.int64)
    h, w, _ = s.shape

    def to8(v):
        if depth == 16:
            return (v >> 8).astype(np.uint8)
        if depth == 8:
            return v.astype(np.uint8)
        return (v * 255 // ((1 << depth) - 1)).astype(np.uint8)

    out = np.zeros((h, w, 4), np.uint8)
    if ctype == 0:
        g = to8(s[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        out[..., 3] = 255
        if trns is not None:
            key = struct.unpack(">H", trns[:2])[0]
            out[..., 3] = np.where(s[..., 0] == key, 0, 255)
    elif ctype == 2:
        for c in range(3):
            out[..., c] = to8(s[..., c])
        out[..., 3] = 255
        if trns is not None:
            key = struct.unpack(">HHH", trns[:6])
            hit = (s[..., 0] == key[0]) & (s[..., 1] == key[1]) & (s[..., 2] == key[2])
            out[..., 3] = np.where(hit, 0, 255)
    elif ctype == 3:
        pal = np.full((len(palette), 4), 255, np.uint8)
        pal[:, :3] = np.asarray(palette, np.uint8)
        if trns is not None:
            pal[:len(trns), 3] = np.frombuffer(trns, np.uint8)
        out[:] = pal[s[..., 0]]
    elif ctype == 4:
        g = to8(s[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        out[..., 3] = to8(s[..., 1])
    else:
        for c in range(4):
            out[..., c] = to8(s[..., c])
    return out
