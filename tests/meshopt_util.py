"""EXT_meshopt_compression encoders for the decoder tests.  Each makes a
valid stream for given data while choosing at random among the encodings
the format allows (group modes and escapes; triangle codes, FIFO hits,
auxiliary-table entries, explicit indices and restarts; sequence baselines),
so that decoding exercises every path.  The triangle encoder checks each
candidate with the oracle's single-triangle step before taking it.  Also the
octahedral / quaternion / exponential filter encoders."""
from __future__ import annotations

import math

import numpy as np

from oracle import meshopt as om

M32 = 0xFFFFFFFF


def varint(v: int) -> bytes:
    out = bytearray()
    while True:
        b, v = v & 0x7F, v >> 7
        out.append(b | (0x80 if v else 0))
        if not v:
            return bytes(out)


def zigzag32(d: int) -> int:
    d = ((d + (1 << 31)) & M32) - (1 << 31)  # as int32
    return ((d << 1) ^ (d >> 31)) & M32


# ------------------------------------------------------------ attributes

def _group(zz: np.ndarray, rng) -> tuple[int, bytes]:
    """A 16-byte group of zig-zag deltas: a random mode that can hold it."""
    modes = ([0] if not zz.any() else []) + [1, 2, 3]
    if rng.random() < 0.5:  # the smallest encoding half of the time
        sizes = {0: 0, 1: 4 + int((zz >= 3).sum()), 2: 8 + int((zz >= 15).sum()), 3: 16}
        mode = min(modes, key=lambda m: sizes[m])
    else:
        mode = modes[int(rng.integers(0, len(modes)))]
    if mode == 0:
        return 0, b""
    if mode == 3:
        return 3, zz.astype(np.uint8).tobytes()
    bits = 2 if mode == 1 else 4
    esc = (1 << bits) - 1
    packed, extra = 0, bytearray()
    for v in zz.tolist():
        code = v if v < esc else esc
        if code == esc:
            extra.append(v)
        packed = (packed << bits) | code
    return mode, packed.to_bytes(2 * bits, "big") + bytes(extra)


def encode_attributes(data: bytes, count: int, stride: int, rng, baseline: bytes | None = None) -> bytes:
    v = np.frombuffer(data, np.uint8, count=count * stride).reshape(count, stride).astype(np.int64)
    if baseline is None:
        baseline = bytes(rng.integers(0, 256, stride, dtype=np.uint8)) if rng.random() < 0.5 else \
            (v[0].astype(np.uint8).tobytes() if count else bytes(stride))
    prev = np.frombuffer(baseline, np.uint8).astype(np.int64).copy()
    block = min((8192 // stride) // 16 * 16, 256)
    out = bytearray([0xA0])
    for first in range(0, count, block):
        n = min(block, count - first)
        groups = (n + 15) // 16
        for k in range(stride):
            col = v[first:first + n, k]
            d = (col - np.concatenate([[prev[k]], col[:-1]])) & 0xFF
            s = np.where(d >= 128, d - 256, d)
            zz = np.where(s >= 0, 2 * s, -2 * s - 1)
            zz = np.concatenate([zz, np.zeros(groups * 16 - n, np.int64)])
            header = bytearray((groups + 3) // 4)
            body = bytearray()
            for g in range(groups):
                mode, payload = _group(zz[16 * g:16 * g + 16], rng)
                header[g // 4] |= mode << (2 * (g % 4))
                body += payload
            out += header + body
            prev[k] = col[-1]
    out += bytes(max(stride, 32) - stride) + baseline
    return bytes(out)


# ------------------------------------------------------------- triangles

def _options(st: om.TriangleState, v: int, nxt: int, explicit: bool, fifo_limit: int) -> list[int]:
    """Auxiliary codes (4 bits) that can produce vertex v as b or c."""
    out = [0] if v == nxt else []
    out += [k for k in range(1, fifo_limit + 1) if st.verts[k - 1] == v]
    if explicit:
        out.append(15)
    return out


def encode_triangles(tris, rng, version: int = 1) -> bytes:
    st = om.TriangleState()
    codes, data = bytearray(), bytearray()
    table: list[int] = []
    for (a, b, c) in tris:
        cands = []  # (code byte, extra data, table aux to add or None)
        for fe in range(15):
            if st.edges[fe] != (a, b):
                continue
            if c == st.next:
                cands.append((fe << 4, b"", None))
            cands += [((fe << 4) | fc, b"", None) for fc in range(1, 13 if version else 15) if st.verts[fc] == c]
            if version and c == (st.last - 1) & M32:
                cands.append(((fe << 4) | 13, b"", None))
            if version and c == (st.last + 1) & M32:
                cands.append(((fe << 4) | 14, b"", None))
            cands.append(((fe << 4) | 15, varint(zigzag32(c - st.last)), None))
        if a == st.next:  # a new: the table codes and 0xFE
            n1 = (st.next + 1) & M32
            for fb in _options(st, b, n1, False, 15):
                n2 = (n1 + 1) & M32 if fb == 0 else n1
                for fc in _options(st, c, n2, False, 15):
                    aux = (fb << 4) | fc
                    if aux in table:
                        cands.append((0xF0 | table.index(aux), b"", None))
                    elif len(table) < 14:
                        cands.append((0xF0 | len(table), b"", aux))
            for fb in _options(st, b, n1, True, 14):
                n2 = (n1 + 1) & M32 if fb == 0 else n1
                for fc in _options(st, c, n2, True, 14):
                    if (fb << 4) | fc == 0:
                        continue  # aux 0 with 0xFE restarts the counter
                    last, extra = st.last, bytearray([(fb << 4) | fc])
                    for f, v in ((fb, b), (fc, c)):
                        if f == 15:
                            extra += varint(zigzag32(v - last))
                            last = v
                    cands.append((0xFE, bytes(extra), None))
        # a explicit (0xFF)
        for fb in _options(st, b, st.next, True, 14):
            n2 = (st.next + 1) & M32 if fb == 0 else st.next
            for fc in _options(st, c, n2, True, 14):
                if (fb << 4) | fc == 0:
                    continue
                extra = bytearray([(fb << 4) | fc]) + varint(zigzag32(a - st.last))
                last = a
                for f, v in ((fb, b), (fc, c)):
                    if f == 15:
                        extra += varint(zigzag32(v - last))
                        last = v
                cands.append((0xFF, bytes(extra), None))
        # restarts: aux 0 sets the new-index counter to 0
        if (a, b, c) == (0, 1, 2):
            cands.append((0xFE, b"\x00", None))
        if (b, c) == (0, 1):
            cands.append((0xFF, b"\x00" + varint(zigzag32(a - st.last)), None))
        ok = []
        for code, extra, aux in cands:
            tbl = bytes(table + ([aux] if aux is not None else []) + [0] * 16)[:16]
            s2 = st.copy()
            got, pos = om.triangle_step(s2, code, extra, 0, tbl, version)
            if got == (a, b, c) and pos == len(extra):
                ok.append((code, extra, aux, s2))
        assert ok, (a, b, c)
        code, extra, aux, s2 = ok[int(rng.integers(0, len(ok)))]
        if aux is not None:
            table.append(aux)
        st = s2
        codes.append(code)
        data += extra
    return bytes([0xE0 | version]) + bytes(codes) + bytes(data) + bytes(table + [0] * (16 - len(table)))


def encode_sequence(indices, rng) -> bytes:
    base = [0, 0]
    out = bytearray([0xD1])
    for i in indices:
        k = int(rng.integers(0, 2))
        out += varint((zigzag32(i - base[k]) << 1) | k)
        base[k] = i & M32
    return bytes(out) + bytes(4)


# ---------------------------------------------------------------- filters

def encode_octahedral(normals: np.ndarray, bits: int, w: np.ndarray, dtype) -> np.ndarray:
    """Unit vectors -> (count, 4) of x, y on the octahedron, z = the encoded
    1.0, w as given."""
    one = (1 << (bits - 1)) - 1
    n = normals / np.abs(normals).sum(1, keepdims=True)
    x, y, z = n[:, 0], n[:, 1], n[:, 2]
    fx = np.where(z < 0, (1 - np.abs(y)) * np.where(x >= 0, 1, -1), x)
    fy = np.where(z < 0, (1 - np.abs(x)) * np.where(y >= 0, 1, -1), y)
    q = np.stack([np.round(fx * one), np.round(fy * one), np.full(len(n), one), w], 1)
    return q.astype(dtype)


def encode_quaternion(q: np.ndarray, bits: int) -> np.ndarray:
    s = (1 << (bits - 1)) - 1
    out = np.zeros((len(q), 4), np.int16)
    for i, v in enumerate(q / np.linalg.norm(q, axis=1, keepdims=True)):
        big = int(np.argmax(np.abs(v)))
        if v[big] < 0:
            v = -v
        for k in range(1, 4):
            out[i, k - 1] = int(round(v[(big + k) & 3] * math.sqrt(2) * s))
        out[i, 3] = (s & ~3) | big
    return out


def encode_exponential(values: np.ndarray, rng) -> np.ndarray:
    """float -> uint32 words of a 24-bit signed mantissa and an 8-bit exponent
    (the value is rounded to 23 significant bits)."""
    out = np.zeros(values.size, np.uint32)
    for i, f in enumerate(values.reshape(-1).astype(np.float64)):
        e = (math.frexp(f)[1] - 23 if f != 0 else 0) + int(rng.integers(0, 2))
        e = max(-100, min(100, e))
        m = int(round(f / 2.0 ** e))
        m = max(-(1 << 23), min((1 << 23) - 1, m))
        out[i] = ((e & 0xFF) << 24) | (m & 0xFFFFFF)
    return out
