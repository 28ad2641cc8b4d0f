"""A JPEG encoder for the decoder tests (ITU-T T.81, sequential or
progressive DCT, Huffman): grey, YCbCr (JFIF) or RGB (Adobe transform 0, or component ids
'R', 'G', 'B'); any sampling factors with integral ratios; 8- or 16-bit
quantisation tables; restart intervals; interleaved or one scan per
component; progressive scan scripts with spectral bands, successive
approximation and end-of-band runs.  Huffman tables are built from the symbol frequencies (lengths
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
           progressive: bool = False, rng=None) -> tuple[bytes, list[np.ndarray]]:
    """image: (H, W) grey or (H, W, 3) RGB uint8.  With `progressive`, a
    SOF2 file whose scan script (DC first and refinement scans, interleaved
    when `interleaved`; AC bands with successive approximation) is drawn
    from `rng`."""
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
        sw, sh = scan_dims[-1]
        mask = np.zeros((bh, bw), bool)
        mask[:sh, :sw] = True
        if single:  # a one-component scan codes only the blocks the image needs
            deq[~mask] = 0
        elif progressive:  # AC scans have one component; DC scans cover the MCUs
            ac = deq.copy()
            ac[..., 0, 0] = 0
            deq[~mask] -= ac[~mask]
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

    if progressive:
        return _write(_progressive_scans(quant, sampling, mcux, mcuy, scan_dims, restart, single, rng), mode, rgb_ids,
                      tables, tq, qt16, ids_for(rgb_ids), h, w, sampling, len(comps), restart, True), expected

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


def ids_for(rgb_ids: bool) -> list[int]:
    return [ord("R"), ord("G"), ord("B")] if rgb_ids else [1, 2, 3]


def _extra(v: int, size: int) -> int:
    return v if v >= 0 else v + (1 << size) - 1


def _progressive_scans(quant, sampling, mcux, mcuy, scan_dims, restart, single, rng):
    """A random valid scan script and each scan's items: ("huff", class,
    table, symbol), ("raw", value, bits) and ("rst",)."""
    nc = len(quant)
    t_of = lambda c: 0 if c == 0 else 1
    scans = []
    al0 = int(rng.integers(0, 3))  # DC point transform, refined down to 0
    dc_groups = [list(range(nc))] if (not single and nc > 1) else [[c] for c in range(nc)]
    script = [("dc", g, 0, 0, 0, al0) for g in dc_groups]
    for c in range(nc):
        a0 = int(rng.integers(0, 3))
        split = int(rng.integers(1, 63))
        script += [("ac", [c], 1, split, 0, a0), ("ac", [c], split + 1, 63, 0, a0)]
        for al in range(a0 - 1, -1, -1):
            if rng.random() < 0.5:
                script.append(("ac", [c], 1, 63, al + 1, al))
            else:
                script += [("ac", [c], 1, split, al + 1, al), ("ac", [c], split + 1, 63, al + 1, al)]
    for al in range(al0 - 1, -1, -1):
        script += [("dc", g, 0, 0, al + 1, al) for g in dc_groups]
    # each coefficient's bits in order: the DC first scans, the AC scans from
    # the highest Al down (first scans before their refinements), then the
    # DC refinements (a stable sort keeps the bands' order)
    script.sort(key=lambda x: (0 if x[0] == "dc" and x[4] == 0 else 2 if x[0] == "dc" else 1, -x[5]))
    zz = ZZ
    for kind, comps_in, ss, se, ah, al in script:
        items = []
        if kind == "dc" and len(comps_in) > 1:
            units = [[(c, [(ux * sampling[c][0] + x, uy * sampling[c][1] + y)
                           for y in range(sampling[c][1]) for x in range(sampling[c][0])]) for c in comps_in]
                     for uy in range(mcuy) for ux in range(mcux)]
        else:
            c = comps_in[0]
            sw, shh = scan_dims[c]
            units = [[(c, [(bx, by)])] for by in range(shh) for bx in range(sw)]
        pred = {c: 0 for c in comps_in}
        eob = {"run": 0, "bits": []}
        cap = int(rng.choice([1, 3, 40, 32767]))

        def flush_eob():
            if eob["run"]:
                r = eob["run"].bit_length() - 1
                items.append(("huff", "ac", t_of(comps_in[0]), r << 4))
                if r:
                    items.append(("raw", eob["run"] - (1 << r), r))
                items.extend(("raw", b, 1) for b in eob["bits"])
                eob["run"], eob["bits"] = 0, []

        for i, unit in enumerate(units):
            if restart and i and i % restart == 0:
                flush_eob()
                items.append(("rst",))
                pred = {c: 0 for c in comps_in}
            for c, coords in unit:
                for (bx, by) in coords:
                    q = [int(v) for v in quant[c][by, bx].reshape(64)]
                    zq = [q[zz[k]] for k in range(64)]
                    if kind == "dc" and ah == 0:
                        v = zq[0] >> al
                        diff = v - pred[c]
                        pred[c] = v
                        sz = _sizes(diff)
                        items.append(("huff", "dc", t_of(c), sz))
                        if sz:
                            items.append(("raw", _extra(diff, sz), sz))
                    elif kind == "dc":
                        items.append(("raw", (zq[0] >> al) & 1, 1))
                    elif ah == 0:
                        vals = [(1 if zq[k] > 0 else -1) * (abs(zq[k]) >> al) for k in range(ss, se + 1)]
                        nz = [j for j, v in enumerate(vals) if v]
                        if not nz:
                            eob["run"] += 1
                            if eob["run"] == cap:
                                flush_eob()
                            continue
                        flush_eob()
                        run = 0
                        for j, v in enumerate(vals[:nz[-1] + 1]):
                            if v == 0:
                                run += 1
                                continue
                            while run > 15:
                                items.append(("huff", "ac", t_of(c), 0xF0))
                                run -= 16
                            sz = _sizes(v)
                            items.append(("huff", "ac", t_of(c), (run << 4) | sz))
                            items.append(("raw", _extra(v, sz), sz))
                            run = 0
                        if nz[-1] < se - ss:
                            eob["run"] = 1
                            if cap == 1:
                                flush_eob()
                    else:
                        # refinement: history = bits above al; corrections for
                        # coefficients already nonzero, new ones as run/size 1
                        events = []  # ("corr", bit) / ("zero",) since the last symbol
                        last_new = -1
                        band = list(range(ss, se + 1))
                        new_pos = [k for k in band if (abs(zq[k]) >> (al + 1)) == 0 and (abs(zq[k]) >> al) == 1]
                        if new_pos:
                            flush_eob()
                        for k in band:
                            a = abs(zq[k]) >> al
                            if (abs(zq[k]) >> (al + 1)) != 0:
                                events.append(("corr", a & 1))
                            elif a == 0:
                                events.append(("zero",))
                            else:
                                while sum(1 for e in events if e[0] == "zero") >= 16:
                                    items.append(("huff", "ac", t_of(c), 0xF0))
                                    zeros = 0
                                    while zeros < 16:
                                        e = events.pop(0)
                                        if e[0] == "zero":
                                            zeros += 1
                                        else:
                                            items.append(("raw", e[1], 1))
                                r = sum(1 for e in events if e[0] == "zero")
                                items.append(("huff", "ac", t_of(c), (r << 4) | 1))
                                items.append(("raw", 1 if zq[k] > 0 else 0, 1))
                                items.extend(("raw", e[1], 1) for e in events if e[0] == "corr")
                                events = []
                                last_new = k
                        if last_new != se:
                            # the rest of the band (its correction bits) joins an end-of-band run
                            eob["run"] += 1
                            eob["bits"].extend(e[1] for e in events if e[0] == "corr")
                            if eob["run"] == cap:
                                flush_eob()
        flush_eob()
        scans.append((comps_in, ss, se, ah, al, items))
    return scans


def _write(scans, mode, rgb_ids, tables, tq, qt16, ids, h, w, sampling, ncomp, restart, progressive) -> bytes:
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
    sof = struct.pack(">BHHB", 8, h, w, ncomp)
    for c in range(ncomp):
        sof += bytes([ids[c], (sampling[c][0] << 4) | sampling[c][1], tq[c]])
    seg(0xC2 if progressive else 0xC0, sof)
    if restart:
        seg(0xDD, struct.pack(">H", restart))
    for comps_in, ss, se, ah, al, items in scans:
        freq = {}
        for it in items:
            if it[0] == "huff":
                d = freq.setdefault((it[1], it[2]), {})
                d[it[3]] = d.get(it[3], 0) + 1
        huff = {k: Table(v) for k, v in freq.items()}
        for (kind, t), table in sorted(huff.items()):
            seg(0xC4, table.segment(0 if kind == "dc" else 1, t))
        sos = bytes([len(comps_in)])
        for c in comps_in:
            t = 0 if c == 0 else 1
            sos += bytes([ids[c], (t << 4) | t])
        seg(0xDA, sos + bytes([ss, se, (ah << 4) | al]))
        bw = BitWriter()
        rst = 0
        for it in items:
            if it[0] == "rst":
                bw.pad()
                bw.out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
            elif it[0] == "huff":
                code, n = huff[(it[1], it[2])].code[it[3]]
                bw.put(code, n)
            else:
                bw.put(it[1], it[2])
        bw.pad()
        out += bw.out
    out += b"\xff\xd9"
    return bytes(out)
