// Zstandard decoder (RFC 8878) for the supercompressed levels of KTX 2.0
// textures (supercompressionScheme 2), which the reference's KTX loader
// (ktx_read, CMakeLists.txt:13) accepts through libktx.  Host code: a level
// is decoded once, before its texels go to the device.
//
// Written from the format specification: frames and skippable frames, raw /
// RLE / compressed blocks, raw / RLE / Huffman-coded (one or four streams,
// with a new or repeated table) literals, and sequences with predefined,
// RLE, FSE-coded or repeated tables, repeat offsets and the optional XXH64
// content checksum.  Dictionaries are refused.  Every read is bounds-checked
// against the input and every write against the output capacity: a corrupt
// or truncated stream returns VKGV_INVALID_ARG, a too-small output
// VKGV_LIMIT_EXCEEDED, never a crash.
#include "vkgv.h"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Fail {
    int code;
};

[[noreturn]] void bad() { throw Fail{VKGV_INVALID_ARG}; }

uint32_t rd_le(const uint8_t* p, int n) {
    uint32_t v = 0;
    for (int i = 0; i < n; ++i) v |= uint32_t(p[i]) << (8 * i);
    return v;
}

int highbit(uint32_t v) {  // index of the highest set bit, v > 0
    int n = 0;
    while (v >>= 1) ++n;
    return n;
}

// ------------------------------------------------------------------ XXH64

constexpr uint64_t kP1 = 0x9E3779B185EBCA87ull, kP2 = 0xC2B2AE3D27D4EB4Full, kP3 = 0x165667B19E3779F9ull,
                   kP4 = 0x85EBCA77C2B2AE63ull, kP5 = 0x27D4EB2F165667C5ull;

uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
uint64_t rd64(const uint8_t* p) {
    uint64_t v;
    std::memcpy(&v, p, 8);
    return v;  // little-endian hosts (x86-64, aarch64)
}
uint64_t xxh_round(uint64_t acc, uint64_t lane) { return rotl(acc + lane * kP2, 31) * kP1; }

uint64_t xxh64(const uint8_t* p, size_t n) {
    const uint8_t* end = p + n;
    uint64_t h;
    if (n >= 32) {
        uint64_t v1 = kP1 + kP2, v2 = kP2, v3 = 0, v4 = 0 - kP1;
        for (; p + 32 <= end; p += 32) {
            v1 = xxh_round(v1, rd64(p));
            v2 = xxh_round(v2, rd64(p + 8));
            v3 = xxh_round(v3, rd64(p + 16));
            v4 = xxh_round(v4, rd64(p + 24));
        }
        h = rotl(v1, 1) + rotl(v2, 7) + rotl(v3, 12) + rotl(v4, 18);
        for (uint64_t v : {v1, v2, v3, v4}) h = (h ^ xxh_round(0, v)) * kP1 + kP4;
    } else {
        h = kP5;
    }
    h += uint64_t(n);
    for (; p + 8 <= end; p += 8) h = rotl(h ^ xxh_round(0, rd64(p)), 27) * kP1 + kP4;
    if (p + 4 <= end) {
        h = rotl(h ^ (uint64_t(rd_le(p, 4)) * kP1), 23) * kP2 + kP3;
        p += 4;
    }
    for (; p < end; ++p) h = rotl(h ^ (uint64_t(*p) * kP5), 11) * kP1;
    h ^= h >> 33;
    h *= kP2;
    h ^= h >> 29;
    h *= kP3;
    h ^= h >> 32;
    return h;
}

// ------------------------------------------------------------ bit readers

// Forward reader (FSE table descriptions): bits from the least significant
// end of each byte, bytes in order.
struct FwdBits {
    const uint8_t* p;
    size_t n, pos = 0;  // pos in bits
    uint32_t get(int k) {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i, ++pos) {
            if ((pos >> 3) >= n) bad();
            v |= uint32_t((p[pos >> 3] >> (pos & 7)) & 1u) << i;
        }
        return v;
    }
    uint32_t peek(int k) {
        const size_t save = pos;
        uint32_t v = 0;
        for (int i = 0; i < k; ++i, ++pos) v |= (((pos >> 3) < n ? (p[pos >> 3] >> (pos & 7)) & 1u : 0u)) << i;
        pos = save;
        return v;
    }
};

// Backward reader (Huffman streams, FSE-coded data): the stream is read from
// its last bit towards its first; the last byte's highest set bit marks the
// end of the padding.  Reads past the first bit return zeros and flag an
// overflow.  A read of k bits takes the k bits below the read position as
// one little-endian window (the first bit read is the value's highest).
struct BackBits {
    const uint8_t* p;
    size_t n;
    int64_t left;  // bits not yet read
    BackBits(const uint8_t* data, size_t size) : p(data), n(size) {
        if (size == 0 || data[size - 1] == 0) bad();
        left = int64_t(size - 1) * 8 + highbit(data[size - 1]);
    }
    // bits [pos, pos + k) of the stream (k <= 32), zeros below bit 0
    uint32_t window(int64_t pos, int k) const {
        if (k == 0) return 0u;
        if (pos < 0) {  // past the first bit: the missing low bits are zeros
            if (pos + k <= 0) return 0u;
            return window(0, int(pos + k)) << int(-pos);
        }
        const size_t byte = size_t(pos >> 3);
        uint64_t v = 0;
        if (byte + 8 <= n) {
            std::memcpy(&v, p + byte, 8);  // little-endian hosts (x86-64, aarch64)
        } else {
            for (size_t i = 0; byte + i < n; ++i) v |= uint64_t(p[byte + i]) << (8 * i);
        }
        return uint32_t((v >> (pos & 7)) & ((uint64_t(1) << k) - 1u));
    }
    uint32_t get(int k) {
        left -= k;
        return window(left, k);
    }
    uint32_t peek(int k) const { return window(left - k, k); }
    bool overflow() const { return left < 0; }
};

// -------------------------------------------------------------------- FSE

struct FseCell {
    uint16_t symbol;
    uint8_t bits;
    uint16_t base;
};

struct FseTable {
    int log = 0;
    std::vector<FseCell> cells;
    bool ok = false;
};

// Decoding table from a normalised distribution (count -1 = "less than 1").
void fse_build(const std::vector<int16_t>& norm, int log, FseTable& t) {
    const uint32_t size = 1u << log;
    t.log = log;
    t.cells.assign(size, FseCell{0, 0, 0});
    std::vector<uint32_t> next(norm.size());
    uint32_t high = size - 1;
    for (size_t s = 0; s < norm.size(); ++s) {
        if (norm[s] == -1) {
            t.cells[high--].symbol = uint16_t(s);
            next[s] = 1;
        } else {
            next[s] = uint32_t(norm[s] > 0 ? norm[s] : 0);
        }
    }
    const uint32_t step = (size >> 1) + (size >> 3) + 3, mask = size - 1;
    uint32_t pos = 0;
    for (size_t s = 0; s < norm.size(); ++s)
        for (int i = 0; i < norm[s]; ++i) {
            t.cells[pos].symbol = uint16_t(s);
            do pos = (pos + step) & mask;
            while (pos > high);
        }
    if (pos != 0) bad();  // the spread must come back to the first cell
    for (uint32_t st = 0; st < size; ++st) {
        const uint16_t s = t.cells[st].symbol;
        const uint32_t x = next[s]++;
        const int nb = log - highbit(x);
        t.cells[st].bits = uint8_t(nb);
        t.cells[st].base = uint16_t((x << nb) - size);
    }
    t.ok = true;
}

// Reads a table description (RFC 8878 4.1.1); returns its size in bytes.
size_t fse_read(const uint8_t* p, size_t n, int max_log, int max_symbol, FseTable& t) {
    FwdBits b{p, n};
    const int log = int(b.get(4)) + 5;
    if (log > max_log) bad();
    int remaining = (1 << log) + 1, threshold = 1 << log, nbits = log + 1;
    std::vector<int16_t> norm;
    bool prev_zero = false;
    while (remaining > 1) {
        if (prev_zero) {
            for (;;) {
                const uint32_t r = b.get(2);
                for (uint32_t i = 0; i < r; ++i) norm.push_back(0);
                if (r != 3) break;
            }
            if ((int)norm.size() > max_symbol) bad();
        }
        const int maxv = (2 * threshold - 1) - remaining;
        int v;
        if ((int)b.peek(nbits - 1) < maxv) {
            v = int(b.get(nbits - 1));
        } else {
            v = int(b.get(nbits));
            if (v >= threshold) v -= maxv;
        }
        const int count = v - 1;
        remaining -= count < 0 ? -count : count;
        norm.push_back(int16_t(count));
        if ((int)norm.size() > max_symbol + 1) bad();
        prev_zero = count == 0;
        while (remaining < threshold && nbits > 1) {
            --nbits;
            threshold >>= 1;
        }
    }
    if (remaining != 1) bad();
    fse_build(norm, log, t);
    return (b.pos + 7) / 8;
}

// ---------------------------------------------------------------- Huffman

struct Huff {
    int max_bits = 0;
    std::vector<uint8_t> sym, len;  // indexed by the max_bits-bit prefix
    bool ok = false;
};

void huff_build(const std::vector<uint8_t>& weights, Huff& h) {
    // the last symbol's weight completes the sum of 2^(w-1) to a power of 2
    uint32_t total = 0;
    for (uint8_t w : weights) {
        if (w > 11) bad();
        if (w) total += 1u << (w - 1);
    }
    if (total == 0) bad();
    const int max_bits = highbit(total) + 1;
    const uint32_t rest = (1u << max_bits) - total;
    if (rest == 0 || (rest & (rest - 1))) bad();
    std::vector<uint8_t> w = weights;
    w.push_back(uint8_t(highbit(rest) + 1));
    if (w.size() > 256 || max_bits > 11) bad();
    h.max_bits = max_bits;
    const uint32_t size = 1u << max_bits;
    h.sym.assign(size, 0);
    h.len.assign(size, 0);
    // codes are assigned from the longest (smallest weight) up: prefixes
    // in increasing weight order, symbols in increasing order within one
    uint32_t pos = 0;
    for (int wt = 1; wt <= max_bits; ++wt)
        for (size_t s = 0; s < w.size(); ++s)
            if (w[s] == wt) {
                const uint32_t span = 1u << (wt - 1);
                const int nb = max_bits + 1 - wt;
                for (uint32_t i = 0; i < span; ++i) {
                    h.sym[pos + i] = uint8_t(s);
                    h.len[pos + i] = uint8_t(nb);
                }
                pos += span;
            }
    if (pos != size) bad();
    h.ok = true;
}

// Huffman tree description (RFC 8878 4.2.1); returns its size in bytes.
size_t huff_read(const uint8_t* p, size_t n, Huff& h) {
    if (n < 1) bad();
    const uint32_t hb = p[0];
    std::vector<uint8_t> w;
    if (hb >= 128) {
        const uint32_t count = hb - 127, bytes = (count + 1) / 2;
        if (1 + bytes > n) bad();
        for (uint32_t i = 0; i < count; ++i) w.push_back(uint8_t(i & 1 ? p[1 + i / 2] & 15 : p[1 + i / 2] >> 4));
        huff_build(w, h);
        return 1 + bytes;
    }
    if (hb == 0 || 1 + hb > n) bad();
    FseTable t;
    const size_t used = fse_read(p + 1, hb, 6, 255, t);
    if (used > hb) bad();
    BackBits b(p + 1 + used, hb - used);
    uint32_t s1 = b.get(t.log), s2 = b.get(t.log);
    for (;;) {
        if (w.size() >= 255) bad();
        const FseCell c1 = t.cells[s1];
        w.push_back(uint8_t(c1.symbol));
        s1 = c1.base + b.get(c1.bits);
        if (b.overflow()) {
            w.push_back(uint8_t(t.cells[s2].symbol));
            break;
        }
        if (w.size() >= 255) bad();
        const FseCell c2 = t.cells[s2];
        w.push_back(uint8_t(c2.symbol));
        s2 = c2.base + b.get(c2.bits);
        if (b.overflow()) {
            w.push_back(uint8_t(t.cells[s1].symbol));
            break;
        }
    }
    huff_build(w, h);
    return 1 + hb;
}

void huff_stream(const uint8_t* p, size_t n, const Huff& h, uint8_t* out, size_t count) {
    BackBits b(p, n);
    for (size_t i = 0; i < count; ++i) {
        const uint32_t k = b.peek(h.max_bits);
        out[i] = h.sym[k];
        b.left -= h.len[k];
    }
    if (b.left != 0) bad();  // a stream ends exactly on its first bit
}

// --------------------------------------------------------------- sequences

constexpr uint32_t kLLBase[36] = {0,  1,  2,  3,  4,  5,   6,   7,   8,   9,    10,   11,   12,   13,    14,    15,    16,   18,
                                  20, 22, 24, 28, 32, 40,  48,  64,  128, 256,  512,  1024, 2048, 4096,  8192,  16384, 32768, 65536};
constexpr uint8_t kLLBits[36] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,  0,  1,  1,
                                 1, 1, 2, 2, 3, 3, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};
constexpr uint32_t kMLBase[53] = {3,  4,  5,  6,  7,  8,  9,  10, 11, 12,  13,  14,  15,  16,   17,   18,   19,   20,
                                  21, 22, 23, 24, 25, 26, 27, 28, 29, 30,  31,  32,  33,  34,   35,   37,   39,   41,
                                  43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051, 4099, 8195, 16387, 32771, 65539};
constexpr uint8_t kMLBits[53] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3, 4, 4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};
// Predefined distributions (RFC 8878 3.1.1.3.2.2).
const std::vector<int16_t> kLLDefault = {4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 2, 2,
                                        2, 2, 2, 2, 2, 2, 2, 3, 2, 1, 1, 1, 1, 1, -1, -1, -1, -1};
const std::vector<int16_t> kMLDefault = {1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                        1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1};
const std::vector<int16_t> kOFDefault = {1, 1, 1, 1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                        1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};

struct FrameState {
    uint8_t* out;
    size_t cap, pos = 0;  // output bytes of this frame so far, from `out`
    uint32_t rep[3] = {1, 4, 8};
    Huff huff;
    FseTable ll, of, ml;
};

// A table of one sequence symbol kind by its compression mode.
size_t seq_table(int mode, const uint8_t* p, size_t n, const std::vector<int16_t>& def, int def_log, int max_log,
                 int max_symbol, FseTable& t) {
    switch (mode) {
        case 0:
            fse_build(def, def_log, t);
            return 0;
        case 1: {
            if (n < 1 || p[0] > max_symbol) bad();
            t.log = 0;
            t.cells.assign(1, FseCell{p[0], 0, 0});
            t.ok = true;
            return 1;
        }
        case 2:
            return fse_read(p, n, max_log, max_symbol, t);
        default:
            if (!t.ok) bad();  // repeat needs a table from an earlier block
            return 0;
    }
}

void put(FrameState& f, const uint8_t* src, size_t n) {
    if (n == 0) return;
    if (n > f.cap - f.pos) throw Fail{VKGV_LIMIT_EXCEEDED};
    std::memcpy(f.out + f.pos, src, n);
    f.pos += n;
}

void compressed_block(FrameState& f, const uint8_t* p, size_t n) {
    // ---- literals
    if (n < 1) bad();
    const uint32_t type = p[0] & 3u, sf = (p[0] >> 2) & 3u;
    size_t regen = 0, csize = 0, hdr = 0;
    std::vector<uint8_t> lit;
    if (type == 0 || type == 1) {
        if (sf == 0 || sf == 2) {
            regen = p[0] >> 3;
            hdr = 1;
        } else if (sf == 1) {
            if (n < 2) bad();
            regen = (p[0] >> 4) | (uint32_t(p[1]) << 4);
            hdr = 2;
        } else {
            if (n < 3) bad();
            regen = (p[0] >> 4) | (uint32_t(p[1]) << 4) | (uint32_t(p[2]) << 12);
            hdr = 3;
        }
        if (type == 0) {
            if (hdr + regen > n) bad();
            lit.assign(p + hdr, p + hdr + regen);
            hdr += regen;
        } else {
            if (hdr + 1 > n) bad();
            lit.assign(regen, p[hdr]);
            hdr += 1;
        }
    } else {
        int streams = sf == 0 ? 1 : 4;
        if (sf <= 1) {
            if (n < 3) bad();
            const uint32_t v = rd_le(p, 3) >> 4;
            regen = v & 0x3FFu;
            csize = v >> 10;
            hdr = 3;
        } else if (sf == 2) {
            if (n < 4) bad();
            const uint32_t v = rd_le(p, 4) >> 4;
            regen = v & 0x3FFFu;
            csize = v >> 14;
            hdr = 4;
        } else {
            if (n < 5) bad();
            const uint64_t v = (uint64_t(rd_le(p, 4)) | (uint64_t(p[4]) << 32)) >> 4;
            regen = size_t(v & 0x3FFFFu);
            csize = size_t(v >> 18);
            hdr = 5;
        }
        if (regen > 128 * 1024 || hdr + csize > n) bad();
        const uint8_t* q = p + hdr;
        size_t qn = csize;
        if (type == 2) {
            f.huff = Huff{};
            const size_t used = huff_read(q, qn, f.huff);
            q += used;
            qn -= used;
        } else if (!f.huff.ok) {
            bad();  // treeless literals reuse the previous block's table
        }
        lit.resize(regen);
        if (streams == 1) {
            huff_stream(q, qn, f.huff, lit.data(), regen);
        } else {
            if (qn < 6) bad();
            const size_t s1 = rd_le(q, 2), s2 = rd_le(q + 2, 2), s3 = rd_le(q + 4, 2);
            if (6 + s1 + s2 + s3 > qn) bad();
            const size_t s4 = qn - 6 - s1 - s2 - s3;
            // the first three streams hold (regen + 3) / 4 literals each, the
            // fourth the rest, which must not be negative
            const size_t per = (regen + 3) / 4;
            if (3 * per > regen) bad();
            const uint8_t* sp = q + 6;
            const size_t sizes[4] = {s1, s2, s3, s4};
            for (int k = 0; k < 4; ++k) {
                const size_t cnt = k < 3 ? per : regen - 3 * per;
                huff_stream(sp, sizes[k], f.huff, lit.data() + k * per, cnt);
                sp += sizes[k];
            }
        }
        hdr += csize;
    }
    // ---- sequences
    const uint8_t* s = p + hdr;
    size_t sn = n - hdr;
    if (sn < 1) bad();
    size_t nseq = s[0], used = 1;
    if (s[0] >= 128 && s[0] < 255) {
        if (sn < 2) bad();
        nseq = ((s[0] - 128u) << 8) + s[1];
        used = 2;
    } else if (s[0] == 255) {
        if (sn < 3) bad();
        nseq = s[1] + (uint32_t(s[2]) << 8) + 0x7F00u;
        used = 3;
    }
    size_t lit_pos = 0;
    if (nseq > 0) {
        if (sn < used + 1) bad();
        const uint8_t modes = s[used++];
        if (modes & 3u) bad();
        used += seq_table(modes >> 6, s + used, sn - used, kLLDefault, 6, 9, 35, f.ll);
        if (used > sn) bad();
        used += seq_table((modes >> 4) & 3, s + used, sn - used, kOFDefault, 5, 8, 31, f.of);
        if (used > sn) bad();
        used += seq_table((modes >> 2) & 3, s + used, sn - used, kMLDefault, 6, 9, 52, f.ml);
        if (used >= sn) bad();
        BackBits b(s + used, sn - used);
        uint32_t sll = b.get(f.ll.log), sof = b.get(f.of.log), sml = b.get(f.ml.log);
        for (size_t i = 0; i < nseq; ++i) {
            const FseCell cll = f.ll.cells[sll], cof = f.of.cells[sof], cml = f.ml.cells[sml];
            const uint32_t ofc = cof.symbol;
            if (ofc > 31 || cll.symbol > 35 || cml.symbol > 52) bad();
            const uint64_t ofv = (uint64_t(1) << ofc) + b.get(int(ofc));
            const size_t ml = kMLBase[cml.symbol] + b.get(kMLBits[cml.symbol]);
            const size_t ll = kLLBase[cll.symbol] + b.get(kLLBits[cll.symbol]);
            // repeat offsets (RFC 8878 3.1.2.5)
            uint64_t off;
            if (ofv > 3) {
                off = ofv - 3;
                f.rep[2] = f.rep[1];
                f.rep[1] = f.rep[0];
                f.rep[0] = uint32_t(off);
            } else {
                const uint32_t idx = uint32_t(ofv - 1) + (ll == 0 ? 1u : 0u);
                if (idx == 0) {
                    off = f.rep[0];
                } else {
                    // the chosen offset moves to the front; offset 3 of a
                    // zero-length literal run is the first one less one
                    off = idx == 3 ? uint64_t(f.rep[0]) - 1 : f.rep[idx];
                    if (idx != 1) f.rep[2] = f.rep[1];
                    f.rep[1] = f.rep[0];
                    f.rep[0] = uint32_t(off);
                }
            }
            if (off == 0) bad();
            // literals, then the match (which may overlap its own output)
            if (ll > lit.size() - lit_pos) bad();
            put(f, lit.data() + lit_pos, ll);
            lit_pos += ll;
            if (off > f.pos) bad();
            if (ml > f.cap - f.pos) throw Fail{VKGV_LIMIT_EXCEEDED};
            uint8_t* d = f.out + f.pos;
            const uint8_t* src = d - off;
            if (off >= 16) {  // 16-byte pieces never overlap their own source
                size_t k = 0;
                for (; k + 16 <= ml; k += 16) std::memcpy(d + k, src + k, 16);
                for (; k < ml; ++k) d[k] = src[k];
            } else {
                for (size_t k = 0; k < ml; ++k) d[k] = src[k];
            }
            f.pos += ml;
            if (i + 1 < nseq) {  // state updates: literal length, match length, offset
                sll = cll.base + b.get(cll.bits);
                sml = cml.base + b.get(cml.bits);
                sof = cof.base + b.get(cof.bits);
            }
        }
        if (b.left != 0) bad();
    }
    put(f, lit.data() + lit_pos, lit.size() - lit_pos);
}

// Decodes one frame at p (n bytes available); returns the bytes it used.
size_t frame(const uint8_t* p, size_t n, uint8_t* out, size_t cap, size_t* written) {
    if (n < 4) bad();
    const uint32_t magic = rd_le(p, 4);
    if ((magic & 0xFFFFFFF0u) == 0x184D2A50u) {  // skippable frame
        if (n < 8) bad();
        const size_t len = rd_le(p + 4, 4);
        if (len > n - 8) bad();
        *written = 0;
        return 8 + len;
    }
    if (magic != 0xFD2FB528u) bad();
    size_t i = 4;
    if (i >= n) bad();
    const uint8_t fhd = p[i++];
    const uint32_t fcs_flag = fhd >> 6, single = (fhd >> 5) & 1u, checksum = (fhd >> 2) & 1u, did = fhd & 3u;
    if (fhd & 0x08u) bad();  // reserved bit
    if (!single) {
        if (i >= n) bad();
        ++i;  // window descriptor: the whole frame is kept, so only checked for presence
    }
    const int did_bytes = did == 0 ? 0 : (did == 1 ? 1 : (did == 2 ? 2 : 4));
    if (i + did_bytes > n) bad();
    if (did_bytes && rd_le(p + i, did_bytes) != 0) bad();  // dictionaries are not supported
    i += did_bytes;
    const int fcs_bytes = fcs_flag == 0 ? (single ? 1 : 0) : (fcs_flag == 1 ? 2 : (fcs_flag == 2 ? 4 : 8));
    if (i + fcs_bytes > n) bad();
    uint64_t fcs = 0;
    bool have_fcs = fcs_bytes > 0;
    if (fcs_bytes == 8) {
        fcs = uint64_t(rd_le(p + i, 4)) | (uint64_t(rd_le(p + i + 4, 4)) << 32);
    } else if (fcs_bytes) {
        fcs = rd_le(p + i, fcs_bytes) + (fcs_bytes == 2 ? 256u : 0u);
    }
    i += fcs_bytes;
    FrameState f;
    f.out = out;
    f.cap = cap;
    for (;;) {
        if (i + 3 > n) bad();
        const uint32_t bh = rd_le(p + i, 3);
        i += 3;
        const uint32_t last = bh & 1u, type = (bh >> 1) & 3u, size = bh >> 3;
        if (type == 3) bad();
        if (type == 1) {
            if (i + 1 > n) bad();
            if (size > f.cap - f.pos) throw Fail{VKGV_LIMIT_EXCEEDED};
            std::memset(f.out + f.pos, p[i], size);
            f.pos += size;
            i += 1;
        } else {
            if (size > 128 * 1024 || i + size > n) bad();
            if (type == 0) put(f, p + i, size);
            else compressed_block(f, p + i, size);
            i += size;
        }
        if (last) break;
    }
    if (have_fcs && fcs != f.pos) bad();
    if (checksum) {
        if (i + 4 > n) bad();
        if (uint32_t(xxh64(f.out, f.pos)) != rd_le(p + i, 4)) bad();
        i += 4;
    }
    *written = f.pos;
    return i;
}

}  // namespace

extern "C" int vkgv_zstd_decompress(const void* src, uint64_t src_size, void* dst, uint64_t dst_capacity,
                                    uint64_t* out_size) {
    if (!src || !out_size || (!dst && dst_capacity)) return VKGV_INVALID_ARG;
    *out_size = 0;
    const uint8_t* p = static_cast<const uint8_t*>(src);
    uint8_t* out = static_cast<uint8_t*>(dst);
    try {
        size_t i = 0, total = 0;
        if (src_size == 0) bad();
        while (i < src_size) {
            size_t w = 0;
            i += frame(p + i, size_t(src_size - i), out + total, size_t(dst_capacity - total), &w);
            total += w;
        }
        *out_size = total;
        return VKGV_OK;
    } catch (const Fail& e) {
        return e.code;
    } catch (...) {
        return VKGV_INVALID_ARG;
    }
}

extern "C" uint64_t vkgv_xxh64(const void* data, uint64_t size) {
    return data || size == 0 ? xxh64(static_cast<const uint8_t*>(data), size_t(size)) : 0u;
}
