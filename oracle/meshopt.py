"""CPU restatement of the EXT_meshopt_compression decoders that the
reference's MeshoptDecompressor::ExecuteRange runs per compressed bufferView
(src/vk_gltf_viewer/assets.cpp:111-166: meshopt_decodeVertexBuffer,
meshopt_decodeIndexBuffer, meshopt_decodeIndexSequence, then
meshopt_decodeFilterOct / Quat / Exp).  TEST INFRASTRUCTURE ONLY: the tests
use it as the checker of the library's decoder, never the product.

meshoptimizer is an empty submodule in the reference (.gitmodules gives only
a URL, no pinned commit), so this follows the bitstream of the published
EXT_meshopt_compression specification; parity with meshoptimizer's own
execution is unpinned.  Pure Python, for streams of a few thousand elements.

Every decoder returns the decoded bytes, or None where the stream is
malformed (a wrong header, data that runs out, or data left over).
"""
from __future__ import annotations

import numpy as np

ATTRIBUTES, TRIANGLES, INDICES = 0, 1, 2
NONE, OCTAHEDRAL, QUATERNION, EXPONENTIAL = 0, 1, 2, 3


def _unzigzag(v: int) -> int:
    """Zig-zag code -> two's-complement delta (as an unsigned 32-bit value)."""
    return ((v >> 1) ^ -(v & 1)) & 0xFFFFFFFF


def _varint(buf: bytes, pos: int) -> tuple[int, int]:
    """Base-128 little-endian varint of at most 5 bytes -> (value, new pos)."""
    value = 0
    for i in range(5):
        b = buf[pos]
        pos += 1
        value |= (b & 0x7F) << (7 * i)
        if b < 0x80:
            break
    return value & 0xFFFFFFFF, pos


def attributes(buf: bytes, count: int, stride: int) -> bytes | None:
    """Mode ATTRIBUTES (header 0xA0): byte columns of zig-zag deltas per
    vertex block, groups of 16 coded in 0 / 2 / 4 / 8 bits, the baseline
    vertex in the stream's last `stride` bytes."""
    if stride <= 0 or stride > 256 or stride % 4 or len(buf) < 1 + stride or buf[0] != 0xA0:
        return None
    prev = list(buf[len(buf) - stride:])
    block = min((8192 // stride) // 16 * 16, 256)
    out = bytearray(count * stride)
    pos = 1
    for first in range(0, count, block):
        n = min(block, count - first)
        groups = (n + 15) // 16
        for k in range(stride):
            header_len = (groups + 3) // 4
            if len(buf) - pos < header_len:
                return None
            header = buf[pos:pos + header_len]
            pos += header_len
            deltas = []
            for g in range(groups):
                if len(buf) - pos < 24:  # room for the largest group
                    return None
                mode = (header[g // 4] >> (2 * (g % 4))) & 3
                if mode == 0:
                    deltas += [0] * 16
                elif mode == 3:
                    deltas += list(buf[pos:pos + 16])
                    pos += 16
                else:
                    bits = 2 if mode == 1 else 4
                    packed = int.from_bytes(buf[pos:pos + 2 * bits], "big")  # first code in the top bits
                    extra = pos + 2 * bits
                    for i in range(16):
                        code = (packed >> (16 * bits - bits * (i + 1))) & ((1 << bits) - 1)
                        if code == (1 << bits) - 1:
                            code = buf[extra]
                            extra += 1
                        deltas.append(code)
                    pos = extra
            v = prev[k]
            for i in range(n):
                d = deltas[i]
                v = (v + ((d >> 1) ^ (0xFF if d & 1 else 0))) & 0xFF
                out[(first + i) * stride + k] = v
            prev[k] = v
    if len(buf) - pos != max(stride, 32):
        return None
    return bytes(out)


def _pack(indices, stride: int) -> bytes:
    dt = "<u2" if stride == 2 else "<u4"
    return np.asarray([i & (0xFFFF if stride == 2 else 0xFFFFFFFF) for i in indices], dtype=dt).tobytes()


class TriangleState:
    """The triangle decoder's state: the edge FIFO and vertex FIFO as lists,
    newest first, 16 entries, initially all 0xFFFFFFFF; the next new index;
    the last explicit index."""

    def __init__(self):
        self.edges = [(0xFFFFFFFF, 0xFFFFFFFF)] * 16
        self.verts = [0xFFFFFFFF] * 16
        self.next = 0
        self.last = 0

    def copy(self) -> "TriangleState":
        s = TriangleState()
        s.edges, s.verts, s.next, s.last = list(self.edges), list(self.verts), self.next, self.last
        return s

    def push_edge(self, a, b):
        self.edges = [(a, b)] + self.edges[:15]

    def push_vert(self, v):
        self.verts = [v] + self.verts[:15]

    def new(self) -> int:
        v = self.next
        self.next = (self.next + 1) & 0xFFFFFFFF
        return v

    def explicit(self, buf: bytes, pos: int) -> tuple[int, int]:
        v, pos = _varint(buf, pos)
        self.last = (self.last + _unzigzag(v)) & 0xFFFFFFFF
        return self.last, pos


def triangle_step(st: TriangleState, code: int, buf: bytes, pos: int, table: bytes,
                  version: int) -> tuple[tuple[int, int, int], int]:
    """Decodes one triangle from its code byte; returns it and the new data
    position (state updated in place)."""
    if code < 0xF0:
        a, b = st.edges[code >> 4]
        fc = code & 15
        if fc == 0:
            c = st.new()
            st.push_vert(c)
        elif fc < (13 if version else 15):
            c = st.verts[fc]
        elif fc == 15:
            c, pos = st.explicit(buf, pos)
            st.push_vert(c)
        else:
            st.last = (st.last + (-1 if fc == 13 else 1)) & 0xFFFFFFFF
            c = st.last
            st.push_vert(c)
        st.push_edge(c, b)
        st.push_edge(a, c)
        return (a, b, c), pos
    if code < 0xFE:
        aux, from_table = table[code & 15], True
    else:
        aux, from_table = buf[pos], False
        pos += 1
        if aux == 0:
            st.next = 0
    fb, fc = aux >> 4, aux & 15
    a = 0 if code == 0xFF else st.new()
    b = st.new() if fb == 0 else st.verts[fb - 1]
    c = st.new() if fc == 0 else st.verts[fc - 1]
    if not from_table:
        if code == 0xFF:
            a, pos = st.explicit(buf, pos)
        if fb == 15:
            b, pos = st.explicit(buf, pos)
        if fc == 15:
            c, pos = st.explicit(buf, pos)
    st.push_vert(a)
    if fb == 0 or (fb == 15 and not from_table):
        st.push_vert(b)
    if fc == 0 or (fc == 15 and not from_table):
        st.push_vert(c)
    st.push_edge(b, a)
    st.push_edge(c, b)
    st.push_edge(a, c)
    return (a, b, c), pos


def triangles(buf: bytes, count: int, stride: int) -> bytes | None:
    """Mode TRIANGLES (header 0xE0 | version, version 0 or 1)."""
    if stride not in (2, 4) or count % 3:
        return None
    tris = count // 3
    if len(buf) < 1 + tris + 16 or buf[0] >> 4 != 0xE or buf[0] & 15 > 1:
        return None
    version = buf[0] & 15
    data_end = len(buf) - 16
    table = buf[data_end:]
    st = TriangleState()
    pos = 1 + tris
    out = []
    for t in range(tris):
        if pos > data_end:
            return None
        tri, pos = triangle_step(st, buf[1 + t], buf, pos, table, version)
        out += tri
    if pos != data_end:
        return None
    return _pack(out, stride)


def sequence(buf: bytes, count: int, stride: int) -> bytes | None:
    """Mode INDICES (header 0xD0 | version): varints whose low bit picks one
    of two baselines and whose remaining bits are a zig-zag delta."""
    if stride not in (2, 4) or len(buf) < 1 + count + 4 or buf[0] >> 4 != 0xD or buf[0] & 15 > 1:
        return None
    data_end = len(buf) - 4
    base = [0, 0]
    pos = 1
    out = []
    for _ in range(count):
        if pos >= data_end:
            return None
        v, pos = _varint(buf, pos)
        base[v & 1] = (base[v & 1] + _unzigzag(v >> 1)) & 0xFFFFFFFF
        out.append(base[v & 1])
    if pos != data_end:
        return None
    return _pack(out, stride)


# ----------------------------------------------------------------- filters
# fp32 arithmetic, one IEEE operation per step in the order written; rounding
# to integers is half away from zero (trunc(v +- 0.5)).

F32 = np.float32


def _round_away(v):
    return np.trunc(np.where(v >= 0, v + F32(0.5), v - F32(0.5))).astype(np.int64)


def octahedral(data: bytes, count: int, stride: int) -> bytes:
    dt = np.int8 if stride == 4 else np.int16
    q = np.frombuffer(data, dtype=dt, count=4 * count).reshape(count, 4).astype(np.int64)
    one = F32((1 << (8 * np.dtype(dt).itemsize - 1)) - 1)
    x, y = q[:, 0].astype(F32), q[:, 1].astype(F32)
    z = (q[:, 2].astype(F32) - np.abs(x)) - np.abs(y)
    fold = np.minimum(z, F32(0))
    x = x + np.where(x >= 0, fold, -fold)
    y = y + np.where(y >= 0, fold, -fold)
    ln = np.sqrt((x * x + y * y) + z * z)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = one / ln
        out = q.copy()
        for i, v in enumerate((x, y, z)):
            out[:, i] = np.where(ln == 0, 0, _round_away(v * s))
    return (out & (0xFF if stride == 4 else 0xFFFF)).astype(np.uint8 if stride == 4 else np.uint16).view(dt).tobytes()


def quaternion(data: bytes, count: int) -> bytes:
    q = np.frombuffer(data, dtype=np.int16, count=4 * count).reshape(count, 4).astype(np.int64)
    inv_sqrt2 = F32(1) / np.sqrt(F32(2))
    s = inv_sqrt2 / (q[:, 3] | 3).astype(F32)
    x, y, z = (q[:, i].astype(F32) * s for i in range(3))
    ww = ((F32(1) - x * x) - y * y) - z * z
    w = np.sqrt(np.maximum(ww, F32(0)))
    largest = q[:, 3] & 3
    out = np.zeros_like(q)
    rows = np.arange(count)
    for k, v in enumerate((x, y, z), start=1):
        out[rows, (largest + k) & 3] = _round_away(v * F32(32767))
    out[rows, largest] = np.trunc(w * F32(32767) + F32(0.5)).astype(np.int64)
    return (out & 0xFFFF).astype(np.uint16).view(np.int16).tobytes()


def exponential(data: bytes, words: int) -> bytes:
    v = np.frombuffer(data, dtype="<u4", count=words).astype(np.int64)
    mantissa = ((v & 0xFFFFFF) ^ 0x800000) - 0x800000
    exponent = ((v >> 24) ^ 0x80) - 0x80
    with np.errstate(over="ignore"):
        return np.ldexp(mantissa.astype(F32), exponent.astype(np.int32)).astype("<f4").tobytes()


def decode(buf: bytes, count: int, stride: int, mode: int, filt: int = NONE) -> bytes | None:
    """One bufferView: decode, then filter (ATTRIBUTES only)."""
    if filt != NONE and mode != ATTRIBUTES:
        return None
    if (filt == OCTAHEDRAL and stride not in (4, 8)) or (filt == QUATERNION and stride != 8):
        return None
    out = {ATTRIBUTES: attributes, TRIANGLES: triangles, INDICES: sequence}[mode](bytes(buf), count, stride)
    if out is None or filt == NONE:
        return out
    if filt == OCTAHEDRAL:
        return octahedral(out, count, stride)
    if filt == QUATERNION:
        return quaternion(out, count)
    return exponential(out, count * stride // 4)
