// JPEG entropy decoding on the host: the first half of a base-colour JPEG
// decode.  The reference links wuffs for JPEG (src/vk_gltf_viewer/
// wuffs_implementation.cpp:1-5, CMakeLists.txt:13) but its image loading is
// an empty task (assets.cpp:467-471), and wuffs is an absent submodule; this
// restates ITU-T T.81 for sequential DCT images with Huffman coding:
//   - SOF0 / SOF1 at 8-bit precision, 1 component (grey) or 3 (YCbCr, or
//     RGB when an Adobe APP14 segment says transform 0 or the component ids
//     are 'R', 'G', 'B'), sampling factors 1-4 with integral ratios to the
//     largest, at most 10 blocks per MCU;
//   - DQT (8- and 16-bit tables), DHT (canonical codes, lengths 1-16), DRI
//     with RST0-7 markers, interleaved scans and single-component scans;
//   - SOF2 progressive images: DC first / refinement scans (interleaved or
//     not) and AC first / refinement scans of spectral bands with
//     end-of-band runs (T.81 G.1.2), coefficients accumulated quantized and
//     multiplied by the table in use at each component's first scan;
//   - lossless, hierarchical and arithmetic-coded images are refused.
// Each block's Huffman-coded DC difference and AC run/size pairs are decoded
// into its natural-order coefficients times the quantisation step, clamped
// to int16; blocks lie in the component's MCU-padded block grid, in raster
// order.  The IDCT, chroma upsampling and colour conversion run on the
// device (texdecode.cu, k_jpeg_idct / k_jpeg_color).  Pinned: a scan that
// reads bits past its entropy data (truncation) is an error, as are a
// missing or out-of-order restart marker and data left before one; bytes
// left after a scan's last block are skipped.
#include "vkgv.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

struct vkgv_jpeg {
    vkgv_jpeg_info info{};
    std::vector<int16_t> coef[3];
};

namespace {

struct JpegError {
    std::string msg;
};
[[noreturn]] void bad(const std::string& m) { throw JpegError{m}; }

// Natural (row-major) index of each zig-zag position: the anti-diagonals of
// the 8x8 block, walked alternately up-right and down-left.
struct ZigZag {
    uint8_t natural[64];
    ZigZag() {
        int k = 0;
        for (int d = 0; d < 15; ++d) {
            const int lo = std::max(0, d - 7), hi = std::min(d, 7);
            if (d % 2 == 0)
                for (int r = hi; r >= lo; --r) natural[k++] = uint8_t(r * 8 + d - r);
            else
                for (int r = lo; r <= hi; ++r) natural[k++] = uint8_t(r * 8 + d - r);
        }
    }
};
const ZigZag& zigzag() {
    static const ZigZag z;
    return z;
}

// A canonical Huffman table: codes of each length in increasing order, in
// the order the values are listed; a 9-bit lookahead table for short codes.
struct Huffman {
    bool defined = false;
    uint8_t fast_len[512];
    uint8_t fast_sym[512];
    int32_t first_code[17], last_code[17], first_index[17];
    uint8_t values[256];

    void build(const uint8_t counts[16], const uint8_t* vals, int total) {
        std::memset(fast_len, 0, sizeof(fast_len));
        std::memcpy(values, vals, size_t(total));
        int32_t code = 0, k = 0;
        for (int len = 1; len <= 16; ++len) {
            first_code[len] = code;
            first_index[len] = k;
            for (int i = 0; i < counts[len - 1]; ++i, ++k, ++code) {
                // an over-subscribed length is refused before its code can
                // index past the lookahead table
                if (code >= (1 << len)) bad("over-subscribed Huffman table");
                if (len <= 9)
                    for (int f = code << (9 - len), e = (code + 1) << (9 - len); f < e; ++f) {
                        fast_len[f] = uint8_t(len);
                        fast_sym[f] = vals[k];
                    }
            }
            last_code[len] = code - 1;  // below first_code when the length is unused
            code <<= 1;
        }
        defined = true;
    }
};

// Bits of one scan's entropy-coded data: stuffed 0xFF 0x00 pairs read as
// 0xFF; a marker (or the end of the input) ends the data, after which zero
// bits are supplied and counted, so that reading them is detected.
struct BitReader {
    const uint8_t* p;
    const uint8_t* end;
    uint64_t acc = 0;
    int n = 0;                   // valid bits in the low end of acc
    uint64_t real_bits = 0;      // bits appended from the data
    uint64_t consumed = 0;       // bits taken
    bool at_marker = false;

    BitReader(const uint8_t* begin, const uint8_t* stop) : p(begin), end(stop) {}

    void fill() {
        while (n <= 56) {
            uint32_t byte = 0;
            if (!at_marker) {
                if (p >= end) {
                    at_marker = true;
                } else if (p[0] != 0xFF) {
                    byte = *p++;
                    real_bits += 8;
                } else if (p + 1 < end && p[1] == 0x00) {
                    byte = 0xFF;
                    p += 2;
                    real_bits += 8;
                } else {
                    at_marker = true;  // p stays on the marker
                }
            }
            acc = (acc << 8) | byte;
            n += 8;
        }
    }
    uint32_t bits(int k) {  // k <= 16
        if (k == 0) return 0;
        if (n < k) fill();
        n -= k;
        consumed += uint64_t(k);
        return uint32_t(acc >> n) & ((1u << k) - 1u);
    }
    int symbol(const Huffman& h) {
        if (n < 16) fill();
        const uint32_t peek = uint32_t(acc >> (n - 9)) & 511u;
        if (h.fast_len[peek]) {
            n -= h.fast_len[peek];
            consumed += h.fast_len[peek];
            return h.fast_sym[peek];
        }
        for (int len = 10; len <= 16; ++len) {
            const int32_t code = int32_t(uint32_t(acc >> (n - len)) & ((1u << len) - 1u));
            if (code >= h.first_code[len] && code <= h.last_code[len]) {
                n -= len;
                consumed += uint64_t(len);
                return h.values[h.first_index[len] + code - h.first_code[len]];
            }
        }
        bad("invalid Huffman code");
    }
    // At a restart or the end of a scan: nothing read past the data; before
    // a restart marker, at most the padding bits of the last byte left over.
    void finish_interval(bool at_restart) {
        if (consumed > real_bits) bad("entropy-coded data ends early");
        if (at_restart && real_bits - consumed >= 8) bad("entropy-coded data longer than its restart interval");
        acc = 0;
        n = 0;
        real_bits = consumed = 0;
    }
};

inline int32_t extend(uint32_t v, int s) {
    return (s && v < (1u << (s - 1))) ? int32_t(v) - (1 << s) + 1 : int32_t(v);
}

inline int16_t clamp16(int64_t v) { return int16_t(std::min<int64_t>(32767, std::max<int64_t>(-32768, v))); }

inline uint32_t be16(const uint8_t* p) { return (uint32_t(p[0]) << 8) | p[1]; }

struct Component {
    uint8_t id = 0, h = 1, v = 1, tq = 0;
    uint32_t blocks_w = 0, blocks_h = 0;  // MCU-padded grid
    uint32_t scan_w = 0, scan_h = 0;      // blocks a single-component scan covers
    bool decoded = false;
};

struct Decoder {
    const uint8_t* data;
    size_t size;
    vkgv_jpeg& out;
    uint16_t qt[4][64];  // zig-zag order
    bool qt_defined[4] = {false, false, false, false};
    Huffman dc[4], ac[4];
    Component comp[3];
    uint32_t ncomp = 0, width = 0, height = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    uint32_t restart = 0;
    bool have_frame = false, adobe = false, progressive = false;
    // progressive: coefficients accumulate quantized over the scans and are
    // multiplied by the table each component's first scan used
    uint16_t latched[3][64];
    bool latched_set[3] = {false, false, false};
    uint8_t adobe_transform = 1;

    Decoder(const uint8_t* d, size_t s, vkgv_jpeg& o) : data(d), size(s), out(o) {}

    void frame(const uint8_t* seg, uint32_t len) {
        if (have_frame) bad("more than one frame header");
        if (len < 6) bad("short frame header");
        if (seg[0] != 8) bad("only 8-bit JPEG is supported");
        height = be16(seg + 1);
        width = be16(seg + 3);
        ncomp = seg[5];
        if (height == 0) bad("JPEG height defined by a DNL marker is not supported");
        if (width == 0) bad("zero-width JPEG");
        if (width > 16384 || height > 16384) bad("JPEG edge exceeds 16384");
        if (ncomp != 1 && ncomp != 3) bad("only 1- or 3-component JPEG is supported");
        if (len < 6 + 3 * ncomp) bad("short frame header");
        for (uint32_t c = 0; c < ncomp; ++c) {
            Component& k = comp[c];
            k.id = seg[6 + 3 * c];
            k.h = seg[7 + 3 * c] >> 4;
            k.v = seg[7 + 3 * c] & 15;
            k.tq = seg[8 + 3 * c];
            if (k.h < 1 || k.h > 4 || k.v < 1 || k.v > 4 || k.tq > 3) bad("bad component in the frame header");
            for (uint32_t d = 0; d < c; ++d)
                if (comp[d].id == k.id) bad("duplicate component id");
            hmax = std::max<uint32_t>(hmax, k.h);
            vmax = std::max<uint32_t>(vmax, k.v);
        }
        uint32_t per_mcu = 0;
        for (uint32_t c = 0; c < ncomp; ++c) {
            if (hmax % comp[c].h || vmax % comp[c].v) bad("non-integral sampling ratio");
            per_mcu += comp[c].h * comp[c].v;
        }
        if (ncomp > 1 && per_mcu > 10) bad("more than 10 blocks per MCU");
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        // every block of the first component takes at least one bit of some
        // scan: a file too small for its frame is refused before the
        // coefficient planes are allocated
        const uint64_t first_blocks = uint64_t((width * comp[0].h + hmax - 1) / hmax + 7) / 8 *
                                      (uint64_t((height * comp[0].v + vmax - 1) / vmax + 7) / 8);
        if (uint64_t(size) * 8 < first_blocks) bad("JPEG data too short for its frame size");
        for (uint32_t c = 0; c < ncomp; ++c) {
            Component& k = comp[c];
            k.blocks_w = mcux * k.h;
            k.blocks_h = mcuy * k.v;
            k.scan_w = ((width * k.h + hmax - 1) / hmax + 7) / 8;
            k.scan_h = ((height * k.v + vmax - 1) / vmax + 7) / 8;
            out.coef[c].assign(size_t(k.blocks_w) * k.blocks_h * 64, 0);
        }
        have_frame = true;
    }

    void tables_q(const uint8_t* seg, uint32_t len) {
        uint32_t at = 0;
        while (at < len) {
            const uint32_t pq = seg[at] >> 4, tq = seg[at] & 15;
            if (pq > 1 || tq > 3) bad("bad quantisation table");
            const uint32_t bytes = pq ? 128 : 64;
            if (at + 1 + bytes > len) bad("short quantisation table");
            for (int k = 0; k < 64; ++k)
                qt[tq][k] = uint16_t(pq ? be16(seg + at + 1 + 2 * k) : seg[at + 1 + k]);
            qt_defined[tq] = true;
            at += 1 + bytes;
        }
    }

    void tables_h(const uint8_t* seg, uint32_t len) {
        uint32_t at = 0;
        while (at < len) {
            if (at + 17 > len) bad("short Huffman table");
            const uint32_t tc = seg[at] >> 4, th = seg[at] & 15;
            if (tc > 1 || th > 3) bad("bad Huffman table class or id");
            int total = 0;
            for (int i = 0; i < 16; ++i) total += seg[at + 1 + i];
            if (total > 256 || at + 17 + uint32_t(total) > len) bad("bad Huffman table size");
            (tc ? ac : dc)[th].build(seg + at + 1, seg + at + 17, total);
            at += 17 + uint32_t(total);
        }
    }

    // Decodes one block into `dst` (64 natural-order coefficients).
    void block(BitReader& br, const Huffman& hd, const Huffman& ha, const uint16_t* q, int32_t& pred, int16_t* dst) {
        const uint8_t* nat = zigzag().natural;
        const int t = br.symbol(hd);
        if (t > 15) bad("DC difference above 15 bits");
        pred = int32_t(uint32_t(pred) + uint32_t(extend(br.bits(t), t)));
        dst[0] = clamp16(int64_t(pred) * q[0]);
        for (int k = 1; k < 64;) {
            const int rs = br.symbol(ha);
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;  // end of block
                k += 16;             // sixteen zeros
                continue;
            }
            k += r;
            if (k > 63) bad("AC coefficients past the end of a block");
            dst[nat[k]] = clamp16(int64_t(extend(br.bits(s), s)) * q[k]);
            ++k;
        }
    }

    // Progressive scans (T.81 G.1.2), on quantized coefficients: a DC scan
    // codes the difference of the point-transformed DC (pred << al) or, when
    // refining, one bit of it; an AC scan codes a spectral band [ss, se] of
    // one component, with end-of-band runs over blocks.
    void dc_first(BitReader& br, const Huffman& hd, int32_t& pred, int al, int16_t* dst) {
        const int t = br.symbol(hd);
        if (t > 15) bad("DC difference above 15 bits");
        pred = int32_t(uint32_t(pred) + uint32_t(extend(br.bits(t), t)));
        dst[0] = clamp16(int64_t(pred) * (int64_t(1) << al));
    }
    static void dc_refine(BitReader& br, int al, int16_t* dst) {
        if (br.bits(1)) dst[0] = int16_t(dst[0] | (1 << al));
    }
    static void ac_first(BitReader& br, const Huffman& ha, int ss, int se, int al, int16_t* dst, uint32_t& eobrun) {
        if (eobrun > 0) {
            --eobrun;
            return;
        }
        const uint8_t* nat = zigzag().natural;
        for (int k = ss; k <= se;) {
            const int rs = br.symbol(ha);
            const int r = rs >> 4, sz = rs & 15;
            if (sz == 0) {
                if (r < 15) {  // this block and (2^r - 1 + r extra bits) more end here
                    eobrun = (1u << r) - 1u + br.bits(r);
                    break;
                }
                k += 16;
                continue;
            }
            k += r;
            if (k > se) bad("AC coefficients past the end of the band");
            dst[nat[k]] = clamp16(int64_t(extend(br.bits(sz), sz)) * (int64_t(1) << al));
            ++k;
        }
    }
    static void ac_refine(BitReader& br, const Huffman& ha, int ss, int se, int al, int16_t* dst, uint32_t& eobrun) {
        const uint8_t* nat = zigzag().natural;
        const int p1 = 1 << al, m1 = -(1 << al);
        // a coefficient already nonzero takes one correction bit
        auto correct = [&](int16_t& c) {
            if (br.bits(1) && (c & p1) == 0) c = clamp16(int32_t(c) + (c >= 0 ? p1 : m1));
        };
        int k = ss;
        if (eobrun == 0) {
            while (k <= se) {
                const int rs = br.symbol(ha);
                int r = rs >> 4;
                const int sz = rs & 15;
                int value = 0;
                if (sz == 0) {
                    if (r < 15) {  // end of band: the rest of this block is refined below
                        eobrun = (1u << r) + br.bits(r);
                        break;
                    }
                    // r = 15: sixteen coefficients still zero are passed
                } else {
                    if (sz != 1) bad("refinement coefficient of more than one bit");
                    value = br.bits(1) ? p1 : m1;
                }
                // pass r coefficients still zero (correcting the nonzero ones
                // on the way), then give the next zero one `value`
                while (k <= se) {
                    int16_t& c = dst[nat[k++]];
                    if (c != 0) {
                        correct(c);
                    } else if (r == 0) {
                        if (value) c = int16_t(value);
                        break;
                    } else {
                        --r;
                    }
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k) {
                int16_t& c = dst[nat[k]];
                if (c != 0) correct(c);
            }
            --eobrun;
        }
    }

    // Returns the position after the scan's entropy-coded data.
    const uint8_t* scan(const uint8_t* seg, uint32_t len, const uint8_t* data_begin, const uint8_t* data_end) {
        if (!have_frame) bad("scan before the frame header");
        if (len < 1) bad("short scan header");
        const uint32_t ns = seg[0];
        if (ns < 1 || ns > ncomp || len < 4 + 2 * ns) bad("bad scan header");
        uint32_t idx[3] = {0, 0, 0};
        const Huffman* hd[3] = {nullptr, nullptr, nullptr};
        const Huffman* ha[3] = {nullptr, nullptr, nullptr};
        uint16_t q[3][64];
        uint32_t per_mcu = 0;
        for (uint32_t i = 0; i < ns; ++i) {
            const uint8_t id = seg[1 + 2 * i];
            uint32_t c = 0;
            while (c < ncomp && comp[c].id != id) ++c;
            if (c == ncomp) bad("scan names an unknown component");
            for (uint32_t j = 0; j < i; ++j)
                if (idx[j] == c) bad("component twice in a scan");
            idx[i] = c;
            const uint32_t td = seg[2 + 2 * i] >> 4, ta = seg[2 + 2 * i] & 15;
            if (td > 3 || ta > 3) bad("bad Huffman table id");
            hd[i] = &dc[td];
            ha[i] = &ac[ta];
            if (!qt_defined[comp[c].tq]) bad("component uses an undefined quantisation table");
            std::memcpy(q[i], qt[comp[c].tq], sizeof(q[i]));
            per_mcu += comp[c].h * comp[c].v;
        }
        if (ns > 1 && per_mcu > 10) bad("more than 10 blocks per MCU");
        const uint8_t* tail = seg + 1 + 2 * ns;
        const int ss = tail[0], se = tail[1], ah = tail[2] >> 4, al = tail[2] & 15;
        if (!progressive) {
            if (ss != 0 || se != 63 || ah != 0 || al != 0) bad("progressive scan parameters in a sequential JPEG");
        } else {
            if (ss > se || se > 63 || ah > 13 || al > 13) bad("bad progressive scan parameters");
            if (ss == 0 && se != 0) bad("a progressive DC scan must code the DC coefficient only");
            if (ss > 0 && ns != 1) bad("a progressive AC scan must have one component");
            if (ah != 0 && ah != al + 1) bad("a refinement scan must add one bit");
        }
        const bool dc_scan = ss == 0, refine = ah != 0;
        for (uint32_t i = 0; i < ns; ++i) {
            if ((!progressive || (dc_scan && !refine)) && !hd[i]->defined) bad("scan uses an undefined Huffman table");
            if ((!progressive || !dc_scan) && !ha[i]->defined) bad("scan uses an undefined Huffman table");
            if (progressive && !latched_set[idx[i]]) {
                std::memcpy(latched[idx[i]], q[i], sizeof(q[i]));
                latched_set[idx[i]] = true;
            }
        }
        const uint32_t units_w = ns == 1 ? comp[idx[0]].scan_w : mcux;
        const uint32_t units_h = ns == 1 ? comp[idx[0]].scan_h : mcuy;
        const uint64_t units = uint64_t(units_w) * units_h;
        ScanPlan S{ns, {idx[0], idx[1], idx[2]}, {hd[0], hd[1], hd[2]}, {ha[0], ha[1], ha[2]}, {}, units_w,
                   ss, se, al, dc_scan, refine, data_end};
        std::memcpy(S.q, q, sizeof(q));
        // restart intervals are independent (predictors and end-of-band runs
        // restart): with many of them, threads decode runs of intervals
        const uint64_t intervals = restart ? (units + restart - 1) / restart : 1;
        const unsigned hw = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
        if (intervals >= 8 && hw > 1 && units * per_mcu >= 4096) {
            std::vector<const uint8_t*> starts;
            if (find_intervals(data_begin, data_end, intervals, starts))
                return decode_parallel(S, units, intervals, starts, std::min<uint64_t>(hw, intervals / 2));
        }
        BitReader br(data_begin, data_end);
        decode_units(br, S, 0, units, 0);
        br.finish_interval(false);
        for (uint32_t i = 0; i < ns; ++i) comp[idx[i]].decoded = true;
        return br.p;
    }

    // What decoding a scan needs besides the bits.
    struct ScanPlan {
        uint32_t ns, idx[3];
        const Huffman* hd[3];
        const Huffman* ha[3];
        uint16_t q[3][64];
        uint32_t units_w;
        int ss, se, al;
        bool dc_scan, refine;
        const uint8_t* data_end;
    };

    // Units [u0, u1) (whole restart intervals), the first one at an interval
    // start; `rst` is the number of the first restart marker expected.
    void decode_units(BitReader& br, const ScanPlan& S, uint64_t u0, uint64_t u1, uint32_t rst) {
        int32_t pred[3] = {0, 0, 0};
        uint32_t eobrun = 0;
        for (uint64_t u = u0; u < u1; ++u) {
            if (restart && u != u0 && u % restart == 0) {
                expect_restart(br, S.data_end, rst);
                rst = (rst + 1) & 7;
                pred[0] = pred[1] = pred[2] = 0;
                eobrun = 0;
            }
            const uint32_t ux = uint32_t(u % S.units_w), uy = uint32_t(u / S.units_w);
            for (uint32_t i = 0; i < S.ns; ++i) {
                Component& k = comp[S.idx[i]];
                const uint32_t bh = S.ns == 1 ? 1 : k.v, bw = S.ns == 1 ? 1 : k.h;
                for (uint32_t y = 0; y < bh; ++y)
                    for (uint32_t x = 0; x < bw; ++x) {
                        const uint32_t gx = ux * bw + x, gy = uy * bh + y;
                        int16_t* dst = out.coef[S.idx[i]].data() + (size_t(gy) * k.blocks_w + gx) * 64;
                        if (!progressive) block(br, *S.hd[i], *S.ha[i], S.q[i], pred[i], dst);
                        else if (S.dc_scan && !S.refine) dc_first(br, *S.hd[i], pred[i], S.al, dst);
                        else if (S.dc_scan) dc_refine(br, S.al, dst);
                        else if (!S.refine) ac_first(br, *S.ha[i], S.ss, S.se, S.al, dst, eobrun);
                        else ac_refine(br, *S.ha[i], S.ss, S.se, S.al, dst, eobrun);
                    }
            }
        }
    }

    // At the end of a restart interval: only padding left, then RST<rst>.
    static void expect_restart(BitReader& br, const uint8_t* data_end, uint32_t rst) {
        br.finish_interval(true);
        if (br.p + 1 >= data_end || br.p[0] != 0xFF || br.p[1] != 0xD0 + rst)
            bad("missing or out-of-order restart marker");
        br.p += 2;
        br.at_marker = false;
    }

    // The start of each restart interval, where the serial reader would find
    // it: after the first 0xFF not followed by 0x00, which must be the next
    // RST marker.  False (the serial decoder then reports the fault) when
    // the markers are missing, out of order or too few.
    static bool find_intervals(const uint8_t* p, const uint8_t* end, uint64_t intervals,
                               std::vector<const uint8_t*>& starts) {
        starts.push_back(p);
        for (uint64_t k = 0; k + 1 < intervals; ++k) {
            for (;;) {
                if (end - p < 2) return false;
                if (p[0] == 0xFF && p[1] != 0x00) break;
                p += p[0] == 0xFF ? 2 : 1;
            }
            if (p[1] != 0xD0 + (k & 7)) return false;
            p += 2;
            starts.push_back(p);
        }
        return true;
    }

    // Runs of whole intervals on `threads` threads; the fault of the first
    // failing run is reported, as the serial decoder would report it.
    const uint8_t* decode_parallel(const ScanPlan& S, uint64_t units, uint64_t intervals,
                                   const std::vector<const uint8_t*>& starts, uint64_t threads) {
        std::vector<std::string> errors(threads);
        std::vector<char> failed(threads, 0);
        const uint8_t* tail = nullptr;
        auto run = [&](uint64_t t) {
            const uint64_t i0 = intervals * t / threads, i1 = intervals * (t + 1) / threads;
            try {
                BitReader br(starts[i0], S.data_end);
                decode_units(br, S, i0 * restart, std::min(units, i1 * restart), uint32_t(i0 & 7));
                if (i1 < intervals) {
                    expect_restart(br, S.data_end, uint32_t((i1 - 1) & 7));
                } else {
                    br.finish_interval(false);
                    tail = br.p;
                }
            } catch (const JpegError& e) {
                errors[t] = e.msg;
                failed[t] = 1;
            } catch (...) {
                errors[t] = "JPEG decode failed";
                failed[t] = 1;
            }
        };
        std::vector<std::thread> pool;
        for (uint64_t t = 1; t < threads; ++t) pool.emplace_back(run, t);
        run(0);
        for (auto& th : pool) th.join();
        for (uint64_t t = 0; t < threads; ++t)
            if (failed[t]) bad(errors[t]);
        for (uint32_t i = 0; i < S.ns; ++i) comp[S.idx[i]].decoded = true;
        return tail;
    }

    void run() {
        if (size < 4 || data[0] != 0xFF || data[1] != 0xD8) bad("not a JPEG file");
        const uint8_t* p = data + 2;
        const uint8_t* end = data + size;
        bool eoi = false;
        while (!eoi) {
            // the next marker, after any fill bytes
            while (p < end && *p != 0xFF) ++p;
            while (p < end && *p == 0xFF) ++p;
            if (p >= end) break;
            const uint8_t m = *p++;
            if (m == 0xD9) {
                eoi = true;
                break;
            }
            if (m == 0x00 || m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) continue;  // stuffing, or no length
            if (end - p < 2) bad("truncated marker segment");
            const uint32_t len = be16(p);
            if (len < 2 || size_t(end - p) < len) bad("truncated marker segment");
            const uint8_t* seg = p + 2;
            const uint32_t body = len - 2;
            p += len;
            switch (m) {
            case 0xC0: case 0xC1: frame(seg, body); break;
            case 0xC2:
                progressive = true;
                frame(seg, body);
                break;
            case 0xC6: case 0xCA: case 0xCE: bad("differential or arithmetic progressive JPEG is not supported");
            case 0xC3: case 0xC5: case 0xC7: case 0xCB: case 0xCF: bad("lossless or hierarchical JPEG is not supported");
            case 0xC9: case 0xCD: case 0xCC: bad("arithmetic-coded JPEG is not supported");
            case 0xC4: tables_h(seg, body); break;
            case 0xDB: tables_q(seg, body); break;
            case 0xDD:
                if (body < 2) bad("short restart interval");
                restart = be16(seg);
                break;
            case 0xDA: p = scan(seg, body, p, end); break;
            case 0xEE:
                if (body >= 12 && std::memcmp(seg, "Adobe", 5) == 0) {
                    adobe = true;
                    adobe_transform = seg[11];
                }
                break;
            default: break;  // APPn, COM, DNL and others carry nothing needed
            }
        }
        if (!have_frame) bad("no frame header");
        for (uint32_t c = 0; c < ncomp; ++c)
            if (!comp[c].decoded) bad("a component has no scan");
        if (progressive) {
            const uint8_t* nat = zigzag().natural;
            for (uint32_t c = 0; c < ncomp; ++c) {
                int16_t* f = out.coef[c].data();
                for (size_t b = 0; b < out.coef[c].size() / 64; ++b, f += 64)
                    for (int k = 0; k < 64; ++k) f[nat[k]] = clamp16(int64_t(f[nat[k]]) * latched[c][k]);
            }
        }
        vkgv_jpeg_info& I = out.info;
        I.width = width;
        I.height = height;
        I.components = ncomp;
        I.rgb = ncomp == 3 && ((adobe && adobe_transform == 0) ||
                               (!adobe && comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B'));
        I.hmax = hmax;
        I.vmax = vmax;
        for (uint32_t c = 0; c < ncomp; ++c) {
            I.h[c] = comp[c].h;
            I.v[c] = comp[c].v;
            I.blocks_w[c] = comp[c].blocks_w;
            I.blocks_h[c] = comp[c].blocks_h;
        }
    }
};

void put_error(char* error, uint32_t cap, const std::string& msg) {
    if (!error || cap == 0) return;
    std::strncpy(error, msg.c_str(), cap - 1);
    error[cap - 1] = '\0';
}

}  // namespace

extern "C" int vkgv_jpeg_decode_coefficients(const void* data, uint64_t size, vkgv_jpeg** out, char* error,
                                             uint32_t error_capacity) {
    if (!data || !out) return VKGV_INVALID_ARG;
    *out = nullptr;
    vkgv_jpeg* j = new (std::nothrow) vkgv_jpeg();
    if (!j) return VKGV_OUT_OF_MEMORY;
    try {
        Decoder(static_cast<const uint8_t*>(data), size_t(size), *j).run();
    } catch (const JpegError& e) {
        put_error(error, error_capacity, e.msg);
        delete j;
        return VKGV_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        put_error(error, error_capacity, "out of host memory");
        delete j;
        return VKGV_OUT_OF_MEMORY;
    }
    *out = j;
    return VKGV_OK;
}

extern "C" int vkgv_jpeg_get_info(const vkgv_jpeg* jpeg, vkgv_jpeg_info* out) {
    if (!jpeg || !out) return VKGV_INVALID_ARG;
    *out = jpeg->info;
    return VKGV_OK;
}

extern "C" int vkgv_jpeg_get_coefficients(const vkgv_jpeg* jpeg, uint32_t component, const int16_t** out) {
    if (!jpeg || !out || component >= jpeg->info.components) return VKGV_INVALID_ARG;
    *out = jpeg->coef[component].data();
    return VKGV_OK;
}

extern "C" void vkgv_jpeg_free(vkgv_jpeg* jpeg) { delete jpeg; }
