"""A baseline JPEG encoder for the decoder tests (ITU-T T.81, sequential DCT,
Huffman): grey, YCbCr (JFIF) or RGB (Adobe transform 0, or component ids
'R', 'G', 'B'); any sampling factors with integral ratios; 8- or 16-bit
quantisation tables; restart intervals; interleaved or one scan per
component.  Huffman tables are built from the symbol frequencies (lengths
limited to 16 by the standard's adjustment, the all-ones code reserved), so
no standard table is needed.  Returns the file and the dequantized
natural-order coefficients the decoder must produce, per component, in the
MCU-padded block grid."""
from __future__ import annotations

import heapq
import math
import struct

import numpy as np


def zigzag_natural() -> list[int]:
    out = []
    for d in range(15):
        lo, hi = max(0, d - 7), min(d, 7)
        rows = range(hi, lo - 1, -1) if d % 2 == 0 else range(lo, hi + 1)
        out += [r * 8 + d - r for r in rows]
    return out


ZZ = zigzag_natural()
_DCT = np.array([[(1 / math.sqrt(2) if u == 0 else 1.0) / 2 * math.cos((2 * x + 1) * u * math.pi / 16)
                  for x in range(8)] for u in range(8)])


def quant_table(quality: int, rng, luma: bool = True) -> np.ndarray:
    """64 steps in natural order: rising with frequency, scaled by quality."""
    u, v = np.meshgrid(np.arange(8), np.arange(8))
    base = 6 + (u + v) * (3 if luma else 5) + rng.integers(0, 4, (8, 8))
    scale = (100 - quality) / 50.0 + 0.02
    return np.clip(np.round(base * scale), 1, 255).astype(np.int64).reshape(64)


def _sizes(v: int) -> int:
    return 0 if v == 0 else int(abs(v)).bit_length()


def _code_lengths(freq: dict[int, int]) -> dict[int, int]:
    """Huffman code lengths, at most 16, with one extra longest code kept
    free (T.81 Annex K.2: a pseudo-symbol reserves the all-ones code)."""
    freq = dict(freq)
    freq[256] = 0  # the reserved code: lowest frequency, listed last
    heap = [(f, i, [s]) for i, (s, f) in enumerate(sorted(freq.items(), key=lambda kv: (kv[1], -kv[0])))]
    heapq.heapify(heap)
    depth = {s: 0 for s in freq}
    if len(heap) == 1:
        depth[heap[0][2][0]] = 1
    tie = len(heap)
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            depth[s] += 1
        heapq.heappush(heap, (f1 + f2, tie, a + b))
        tie += 1
    bits = [0] * 33
    for s, d in depth.items():
        bits[d] += 1
    # Annex K.3 (Figure K.3): move codes longer than 16 up the tree
    for i in range(32, 16, -1):
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
    # hand the lengths out again, shortest codes to the most frequent symbols
    order = sorted(freq, key=lambda s: (-freq[s], s == 256, s))
    order.remove(256)
    order.append(256)
    lengths, k = {}, 0
    for length in range(1, 17):
        for _ in range(bits[length]):
            lengths[order[k]] = length
            k += 1
    del lengths[256]
    return lengths


class Table:
    def __init__(self, freq: dict[int, int]):
        lengths = _code_lengths(freq)
        self.values = sorted(lengths, key=lambda s: (lengths[s], s))
        self.counts = [sum(1 for s in self.values if lengths[s] == n) for n in range(1, 17)]
        self.code = {}
        code, k = 0, 0
        for n in range(1, 17):
            for _ in range(self.counts[n - 1]):
                self.code[self.values[k]] = (code, n)
                code += 1
                k += 1
            code <<= 1

    def segment(self, tc: int, th: int) -> bytes:
        return bytes([(tc << 4) | th] + self.counts + self.values)


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, n: int):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def pad(self):
        while self.n:
            self.put(1, 1)


def _blocks(plane: np.ndarray, bw: int, bh: int) -> np.ndarray:
    """Edge-replicated plane -> (bh, bw, 8, 8) level-shifted float blocks."""
    h, w = plane.shape
    p = np.pad(plane.astype(np.float64), ((0, bh * 8 - h), (0, bw * 8 - w)), mode="edge") - 128.0
    return p.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)


def encode(image: np.ndarray, mode: str = "ycc", sampling=((1, 1), (1, 1), (1, 1)), quality: int = 90,
           restart: int = 0, interleaved: bool = True, rgb_ids: bool = False, qt16: bool = False,
           rng=None) -> tuple[bytes, list[np.ndarray]]:
    """image: (H, W) grey or (H, W, 3) RGB uint8."""
    rng = rng or np.random.default_rng(0)
    img = np.asarray(image, np.float64)
    h, w = img.shape[:2]
    if mode == "gray":
        comps, sampling = [img if img.ndim == 2 else img[..., 0]], sampling[:1]
    elif mode == "ycc":
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        comps = [0.299 * r + 0.587 * g + 0.114 * b, -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
                 0.5 * r - 0.418688 * g - 0.081312 * b + 128]
    else:
        comps = [img[..., k] for k in range(3)]
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    tables = [quant_table(quality, rng, True), quant_table(quality, rng, False)]
    if qt16:
        tables = [np.minimum(t * 3 + 1, 60000) for t in tables]
    tq = [0] + [1] * (len(comps) - 1)
    quant, expected, scan_dims = [], [], []
    single = not interleaved or len(comps) == 1
    for c, plane in enumerate(comps):
        hc, vc = sampling[c]
        cw, ch = -(-w * hc // hmax), -(-h * vc // vmax)
        rx, ry = hmax // hc, vmax // vc
        # box-subsample (any resampling will do: the test checks the decoder
        # against the coefficients written)
        pp = np.pad(plane, ((0, ch * ry - h), (0, cw * rx - w)), mode="edge")
        sub = np.clip(np.round(pp.reshape(ch, ry, cw, rx).mean((1, 3))), 0, 255)
        bw, bh = mcux * hc, mcuy * vc
        coef = np.einsum("ux,vy,abyx->abvu", _DCT, _DCT, _blocks(sub, bw, bh))
        q = tables[tq[c]].reshape(8, 8)
        qc = np.round(coef / q).astype(np.int64)
        quant.append(qc)
        deq = np.clip(qc * q, -32768, 32767).astype(np.int16)
        scan_dims.append((-(-cw // 8), -(-ch // 8)))
        if single:  # a one-component scan codes only the blocks the image needs
            sw, sh = scan_dims[-1]
            mask = np.zeros((bh, bw), bool)
            mask[:sh, :sw] = True
            deq[~mask] = 0
        expected.append(deq)

    def block_symbols(qc, pred):
        zz = [int(qc.reshape(64)[ZZ[k]]) for k in range(64)]
        syms = []
        diff = zz[0] - pred
        s = _sizes(diff)
        syms.append(("dc", s, diff, s))
        run = 0
        last = max([k for k in range(1, 64) if zz[k]] or [0])
        for k in range(1, last + 1):
            if zz[k] == 0:
                run += 1
                continue
            while run > 15:
                syms.append(("ac", 0xF0, 0, 0))
                run -= 16
            s = _sizes(zz[k])
            syms.append(("ac", (run << 4) | s, zz[k], s))
            run = 0
        if last < 63:
            syms.append(("ac", 0x00, 0, 0))
        return syms, zz[0]

    # scans: lists of (component, block coordinates) per MCU
    if not single:
        scans = [[(c, [(ux * sampling[c][0] + x, uy * sampling[c][1] + y)
                       for y in range(sampling[c][1]) for x in range(sampling[c][0])])
                  for c in range(len(comps))] for uy in range(mcuy) for ux in range(mcux)]
        scan_list = [(list(range(len(comps))), scans)]
    else:
        scan_list = []
        for c in range(len(comps)):
            sw, sh = scan_dims[c]
            scan_list.append(([c], [[(c, [(bx, by)])] for by in range(sh) for bx in range(sw)]))

    # symbols per scan, then tables from all frequencies
    coded = []
    freq = {("dc", 0): {}, ("ac", 0): {}, ("dc", 1): {}, ("ac", 1): {}}
    for comps_in, units in scan_list:
        seq = []
        pred = {c: 0 for c in comps_in}
        for i, unit in enumerate(units):
            if restart and i and i % restart == 0:
                seq.append(("rst",))
                pred = {c: 0 for c in comps_in}
            for c, coords in unit:
                for (bx, by) in coords:
                    syms, pred[c] = block_symbols(quant[c][by, bx], pred[c])
                    for kind, sym, val, size in syms:
                        d = freq[(kind, 0 if c == 0 else 1)]
                        d[sym] = d.get(sym, 0) + 1
                        seq.append((kind, 0 if c == 0 else 1, sym, val, size))
        coded.append((comps_in, seq))
    huff = {k: Table(v) for k, v in freq.items() if v}

    out = bytearray(b"\xff\xd8")

    def seg(marker: int, body: bytes):
        out.extend(struct.pack(">BBH", 0xFF, marker, len(body) + 2) + body)

    if mode == "rgb" and not rgb_ids:
        seg(0xEE, b"Adobe" + struct.pack(">HHHB", 100, 0, 0, 0))
    elif mode != "rgb":
        seg(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    for t in sorted(set(tq)):
        vals = [int(tables[t][ZZ[k]]) for k in range(64)]
        if qt16:
            seg(0xDB, bytes([0x10 | t]) + struct.pack(">64H", *vals))
        else:
            seg(0xDB, bytes([t] + vals))
    ids = [ord("R"), ord("G"), ord("B")] if rgb_ids else [1, 2, 3]
    sof = struct.pack(">BHHB", 8, h, w, len(comps))
    for c in range(len(comps)):
        sof += bytes([ids[c], (sampling[c][0] << 4) | sampling[c][1], tq[c]])
    seg(0xC0, sof)
    for (kind, t), table in sorted(huff.items()):
        seg(0xC4, table.segment(0 if kind == "dc" else 1, t))
    if restart:
        seg(0xDD, struct.pack(">H", restart))
    for comps_in, seq in coded:
        sos = bytes([len(comps_in)])
        for c in comps_in:
            t = 0 if c == 0 else 1
            sos += bytes([ids[c], (t << 4) | t])
        seg(0xDA, sos + b"\x00\x3f\x00")
        bw_ = BitWriter()
        rst = 0
        for item in seq:
            if item[0] == "rst":
                bw_.pad()
                bw_.out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
                continue
            kind, t, sym, val, size = item
            code, n = huff[(kind, t)].code[sym]
            bw_.put(code, n)
            if size:
                bw_.put(val if val >= 0 else val + (1 << size) - 1, size)
        bw_.pad()
        out += bw_.out
    out += b"\xff\xd9"
    return bytes(out), expected
