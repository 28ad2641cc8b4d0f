// Image containers for base-colour textures: PNG into RGBA8 on the host
// (DEFLATE per RFC 1951 inside the zlib wrapper of RFC 1950, then the PNG
// filters and Adam7 interlacing of the PNG specification), and the DDS
// header (with its DX10 extension) that locates block-compressed data for
// the device decoder.  The reference's image loading is an empty task
// (src/vk_gltf_viewer/assets.cpp:467-471) over wuffs / dds_image / KTX; this
// is an own implementation of the published formats.  Host code, run once
// per texture.
#include "vkgv.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

struct vkgv_image {
    std::vector<uint8_t> rgba;
    uint32_t width = 0, height = 0;
};

namespace {

struct DecodeError {
    const char* msg;
};

[[noreturn]] void fail(const char* m) { throw DecodeError{m}; }

// ------------------------------------------------------------- inflate

class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    uint32_t bits(int k) {  // LSB-first
        while (cnt_ < k) {
            if (pos_ >= n_) fail("DEFLATE stream is truncated");
            acc_ |= uint64_t(p_[pos_++]) << cnt_;
            cnt_ += 8;
        }
        const uint32_t v = uint32_t(acc_ & ((1ull << k) - 1));
        acc_ >>= k;
        cnt_ -= k;
        return v;
    }
    // The next k bits without taking them; past the end of the stream the
    // missing bits read as zeros (taking them then fails).
    uint32_t peek(int k) {
        while (cnt_ <= 56 && pos_ < n_) {
            acc_ |= uint64_t(p_[pos_++]) << cnt_;
            cnt_ += 8;
        }
        return uint32_t(acc_ & ((1ull << k) - 1));
    }
    void consume(int k) {
        if (k > cnt_) fail("DEFLATE stream is truncated");
        acc_ >>= k;
        cnt_ -= k;
    }
    void align() {
        acc_ >>= cnt_ & 7;
        cnt_ -= cnt_ & 7;
    }
    size_t byte_pos() const { return pos_ - size_t(cnt_ / 8); }
    const uint8_t* data() const { return p_; }
    size_t size() const { return n_; }
    void skip_to(size_t byte) {
        pos_ = byte;
        acc_ = 0;
        cnt_ = 0;
    }

private:
    const uint8_t* p_;
    size_t n_, pos_ = 0;
    uint64_t acc_ = 0;
    int cnt_ = 0;
};

// Canonical Huffman code (RFC 1951 3.2.2): codes of each length are
// consecutive, starting at next_code[len] as the RFC assigns them.  Codes of
// at most kFastBits bits decode with one lookup of the next kFastBits stream
// bits (the code is stored most-significant bit first, so the table is
// indexed by its bit-reversed form, every value of the bits after it filled
// in); longer codes are read one bit at a time, checking at each length
// whether the code read so far falls in that length's range.
constexpr int kFastBits = 10;
struct Huffman {
    int32_t first[16] = {};   // first code of each length
    int32_t count[16] = {};   // codes of each length
    int32_t offset[16] = {};  // index in `symbol` of each length's first code
    std::vector<uint16_t> symbol;  // symbols ordered by (length, value)
    uint16_t fast[1 << kFastBits] = {};  // symbol << 4 | length, 0 = a longer code

    void build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int32_t code = 0, slots = 1, idx = 0;
        for (int len = 1; len < 16; ++len) {
            code = (code + count[len - 1]) << 1;  // RFC 1951 3.2.2 step 2
            first[len] = code;
            offset[len] = idx;
            idx += count[len];
            slots = (slots << 1) - count[len];
            if (slots < 0) fail("over-subscribed Huffman code");
        }
        symbol.assign(size_t(idx), 0);
        std::vector<int32_t> fill(offset, offset + 16);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[size_t(fill[lengths[i]]++)] = uint16_t(i);
        std::memset(fast, 0, sizeof(fast));
        for (int len = 1; len <= kFastBits; ++len)
            for (int32_t k = 0; k < count[len]; ++k) {
                const uint32_t code = uint32_t(first[len] + k);
                uint32_t rev = 0;
                for (int b = 0; b < len; ++b) rev |= ((code >> b) & 1u) << (len - 1 - b);
                const uint16_t e = uint16_t((uint32_t(symbol[size_t(offset[len] + k)]) << 4) | uint32_t(len));
                for (uint32_t f = rev; f < (1u << kFastBits); f += 1u << len) fast[f] = e;
            }
    }

    int decode(BitReader& br) const {
        const uint16_t e = fast[br.peek(kFastBits)];
        if (e) {
            br.consume(e & 15);
            return e >> 4;
        }
        int32_t code = 0;
        for (int len = 1; len < 16; ++len) {
            code = (code << 1) | int32_t(br.bits(1));
            const int32_t k = code - first[len];
            if (k >= 0 && k < count[len]) return symbol[size_t(offset[len] + k)];
        }
        fail("invalid Huffman code");
    }
};

// Length and distance bases and extra bits (RFC 1951 3.2.5).
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order of the code-length code lengths (RFC 1951 3.2.7).
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// Inflated bytes: out[0, pos), the vector grown by doubling up to `limit`.
struct Output {
    std::vector<uint8_t> buf;
    size_t pos = 0, limit = 0;
    uint8_t* room(size_t n) {
        if (n > limit - pos) fail("inflated data exceeds the image size");
        if (pos + n > buf.size()) buf.resize(std::min(limit, std::max(pos + n, 2 * buf.size())));
        return buf.data() + pos;
    }
};

void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, Output& out) {
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 256) {
            *out.room(1) = uint8_t(sym);
            ++out.pos;
        } else if (sym == 256) {
            return;
        } else {
            const int li = sym - 257;
            if (li >= 29) fail("invalid length symbol");
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int di = dist.decode(br);
            if (di >= 30) fail("invalid distance symbol");
            const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
            if (d > out.pos) fail("distance beyond the start of the output");
            uint8_t* o = out.room(len);
            const uint8_t* from = o - d;
            for (size_t k = 0; k < len; ++k) o[k] = from[k];  // may overlap its own output
            out.pos += len;
        }
    }
}

// zlib (RFC 1950) around DEFLATE; `limit` bounds the output.
std::vector<uint8_t> zlib_inflate(const uint8_t* data, size_t size, size_t limit) {
    if (size < 6) fail("zlib stream is truncated");
    const uint8_t cmf = data[0], flg = data[1];
    if ((cmf & 15) != 8 || ((uint32_t(cmf) << 8) | flg) % 31 != 0) fail("not a zlib DEFLATE stream");
    if (flg & 0x20) fail("zlib preset dictionaries are not supported");
    BitReader br(data + 2, size - 2);
    Output out;
    out.limit = limit;
    // DEFLATE expands at most about 1032:1 (258-byte matches coded in 2 bits),
    // so a small stream cannot claim a huge buffer up front
    out.buf.resize(std::min(limit, size * 1032 + 1024));
    int last = 0;
    while (!last) {
        last = int(br.bits(1));
        const uint32_t type = br.bits(2);
        if (type == 0) {
            br.align();
            const uint32_t len = br.bits(16), nlen = br.bits(16);
            if ((len ^ 0xFFFFu) != nlen) fail("stored block length mismatch");
            const size_t at = br.byte_pos();
            if (at + len > br.size()) fail("stored block is truncated");
            if (len) std::memcpy(out.room(len), br.data() + at, len);
            out.pos += len;
            br.skip_to(at + len);
        } else if (type == 1) {
            // the fixed codes of RFC 1951 3.2.6, built once (thread-safely)
            struct Fixed {
                Huffman lit, dist;
                Fixed() {
                    uint8_t l[288], d[30];
                    for (int i = 0; i < 144; ++i) l[i] = 8;
                    for (int i = 144; i < 256; ++i) l[i] = 9;
                    for (int i = 256; i < 280; ++i) l[i] = 7;
                    for (int i = 280; i < 288; ++i) l[i] = 8;
                    for (int i = 0; i < 30; ++i) d[i] = 5;
                    lit.build(l, 288);
                    dist.build(d, 30);
                }
            };
            static const Fixed fixed;
            inflate_block(br, fixed.lit, fixed.dist, out);
        } else if (type == 2) {
            const int hlit = int(br.bits(5)) + 257, hdist = int(br.bits(5)) + 1, hclen = int(br.bits(4)) + 4;
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = uint8_t(br.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {};
            int n = 0;
            while (n < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 16) {
                    lens[n++] = uint8_t(sym);
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (n == 0) fail("repeat with no previous length");
                        val = lens[n - 1];
                        rep = 3 + int(br.bits(2));
                    } else if (sym == 17) {
                        rep = 3 + int(br.bits(3));
                    } else {
                        rep = 11 + int(br.bits(7));
                    }
                    if (n + rep > hlit + hdist) fail("code lengths overflow");
                    while (rep--) lens[n++] = val;
                }
            }
            if (lens[256] == 0) fail("no end-of-block code");
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            fail("reserved DEFLATE block type");
        }
    }
    // Adler-32 of the output (RFC 1950 2.2), after the last byte
    br.align();
    const size_t at = br.byte_pos() + 2;
    if (at + 4 > size) fail("zlib checksum is missing");
    out.buf.resize(out.pos);
    // the sums are reduced every 5552 bytes, the most that keeps b in 32 bits
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < out.pos;) {
        const size_t end = std::min(out.pos, i + 5552);
        for (; i < end; ++i) {
            a += out.buf[i];
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
    }
    const uint32_t want = (uint32_t(data[at]) << 24) | (uint32_t(data[at + 1]) << 16) | (uint32_t(data[at + 2]) << 8) |
                          uint32_t(data[at + 3]);
    if (((b << 16) | a) != want) fail("zlib checksum mismatch");
    return std::move(out.buf);
}

// ------------------------------------------------------------------ PNG

uint32_t be32(const uint8_t* p) {
    return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}

// CRC-32 of PNG chunks (the reflected polynomial 0xEDB88320).
uint32_t crc32(const uint8_t* p, size_t n) {
    struct Table {
        uint32_t t[256];
        Table() {
            for (uint32_t i = 0; i < 256; ++i) {
                uint32_t c = i;
                for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
                t[i] = c;
            }
        }
    };
    static const Table tab;
    const uint32_t* table = tab.t;
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return uint8_t(a);
    return uint8_t(pb <= pc ? b : c);
}

// Reverses the per-scanline filters of one (sub)image in place: one loop
// per filter type, the first pixel's bytes (no left neighbour) apart.
void unfilter(uint8_t* data, uint32_t rows, size_t stride, size_t bpp) {
    std::vector<uint8_t> zero(stride, 0);
    const size_t head = std::min(bpp, stride);
    for (uint32_t y = 0; y < rows; ++y) {
        uint8_t* line = data + size_t(y) * (stride + 1);
        const uint8_t ft = line[0];
        uint8_t* cur = line + 1;
        const uint8_t* prev = y ? data + size_t(y - 1) * (stride + 1) + 1 : zero.data();
        switch (ft) {
            case 0:
                break;
            case 1:
                for (size_t i = bpp; i < stride; ++i) cur[i] = uint8_t(cur[i] + cur[i - bpp]);
                break;
            case 2:
                for (size_t i = 0; i < stride; ++i) cur[i] = uint8_t(cur[i] + prev[i]);
                break;
            case 3:
                for (size_t i = 0; i < head; ++i) cur[i] = uint8_t(cur[i] + (prev[i] >> 1));
                for (size_t i = bpp; i < stride; ++i) cur[i] = uint8_t(cur[i] + ((cur[i - bpp] + prev[i]) >> 1));
                break;
            case 4:
                for (size_t i = 0; i < head; ++i) cur[i] = uint8_t(cur[i] + prev[i]);  // paeth(0, b, 0) = b
                for (size_t i = bpp; i < stride; ++i) cur[i] = uint8_t(cur[i] + paeth(cur[i - bpp], prev[i], prev[i - bpp]));
                break;
            default:
                fail("unknown PNG filter type");
        }
    }
}

struct PngInfo {
    uint32_t w, h;
    int depth, ctype, channels;
    std::vector<uint8_t> palette;  // RGBA per entry
    bool has_key = false;
    uint16_t key[3] = {0, 0, 0};   // tRNS colour key (gray or RGB)
};

// Sample k of a row of `bits`-deep samples.
uint32_t sample(const uint8_t* row, size_t k, int bits) {
    if (bits == 8) return row[k];
    if (bits == 16) return (uint32_t(row[2 * k]) << 8) | row[2 * k + 1];
    const size_t bit = k * size_t(bits);
    return (row[bit >> 3] >> (8 - bits - int(bit & 7))) & ((1u << bits) - 1);
}

// One pixel to RGBA8: 16-bit samples keep their high byte, 1/2/4-bit gray
// is scaled by 255 / (2^d - 1), palette entries carry tRNS alpha.
void put_pixel(const PngInfo& I, const uint8_t* row, uint32_t x, uint8_t* dst) {
    const int d = I.depth;
    auto to8 = [&](uint32_t v) -> uint8_t {
        if (d == 16) return uint8_t(v >> 8);
        if (d == 8) return uint8_t(v);
        return uint8_t(v * 255u / ((1u << d) - 1u));
    };
    const size_t k = size_t(x) * size_t(I.channels);
    switch (I.ctype) {
        case 0: {
            const uint32_t g = sample(row, k, d);
            dst[0] = dst[1] = dst[2] = to8(g);
            dst[3] = (I.has_key && g == I.key[0]) ? 0 : 255;
            break;
        }
        case 2: {
            const uint32_t r = sample(row, k, d), g = sample(row, k + 1, d), b = sample(row, k + 2, d);
            dst[0] = to8(r), dst[1] = to8(g), dst[2] = to8(b);
            dst[3] = (I.has_key && r == I.key[0] && g == I.key[1] && b == I.key[2]) ? 0 : 255;
            break;
        }
        case 3: {
            const uint32_t i = sample(row, k, d);
            if (size_t(i) * 4 + 3 >= I.palette.size()) fail("palette index out of range");
            std::memcpy(dst, &I.palette[size_t(i) * 4], 4);
            break;
        }
        case 4:
            dst[0] = dst[1] = dst[2] = to8(sample(row, k, d));
            dst[3] = to8(sample(row, k + 1, d));
            break;
        default:
            for (int c = 0; c < 4; ++c) dst[c] = to8(sample(row, k + size_t(c), d));
    }
}

void decode_png(const uint8_t* p, size_t n, vkgv_image& img) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n < 8 || std::memcmp(p, sig, 8) != 0) fail("not a PNG file");
    PngInfo I{};
    bool have_hdr = false, done = false;
    int interlace = 0;
    std::vector<uint8_t> idat;
    size_t at = 8;
    while (at + 12 <= n && !done) {
        const uint32_t len = be32(p + at);
        if (len > n - at - 12) fail("PNG chunk exceeds the file");
        const uint8_t* type = p + at + 4;
        const uint8_t* data = p + at + 8;
        if (crc32(type, size_t(len) + 4) != be32(data + len)) fail("PNG chunk CRC mismatch");
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) fail("bad IHDR");
            I.w = be32(data);
            I.h = be32(data + 4);
            I.depth = data[8];
            I.ctype = data[9];
            interlace = data[12];
            if (data[10] != 0 || data[11] != 0 || interlace > 1) fail("unsupported PNG compression, filter or interlace");
            static const int ch[7] = {1, 0, 3, 1, 2, 0, 4};
            if (I.ctype > 6 || ch[I.ctype] == 0) fail("bad PNG colour type");
            I.channels = ch[I.ctype];
            const bool ok = (I.ctype == 0 && (I.depth == 1 || I.depth == 2 || I.depth == 4 || I.depth == 8 ||
                                             I.depth == 16)) ||
                            (I.ctype == 3 && (I.depth == 1 || I.depth == 2 || I.depth == 4 || I.depth == 8)) ||
                            ((I.ctype == 2 || I.ctype == 4 || I.ctype == 6) && (I.depth == 8 || I.depth == 16));
            if (!ok) fail("bad PNG bit depth for its colour type");
            if (I.w == 0 || I.h == 0 || I.w > 16384 || I.h > 16384) fail("PNG size out of range");
            have_hdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            if (len % 3 || len > 768) fail("bad PLTE");
            I.palette.assign(size_t(len / 3) * 4, 255);
            for (uint32_t i = 0; i < len / 3; ++i) std::memcpy(&I.palette[i * 4], data + 3 * i, 3);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            if (I.ctype == 3) {
                for (uint32_t i = 0; i < len && size_t(i) * 4 + 3 < I.palette.size(); ++i) I.palette[i * 4 + 3] = data[i];
            } else if (I.ctype == 0 && len >= 2) {
                I.has_key = true;
                I.key[0] = uint16_t((data[0] << 8) | data[1]);
            } else if (I.ctype == 2 && len >= 6) {
                I.has_key = true;
                for (int c = 0; c < 3; ++c) I.key[c] = uint16_t((data[2 * c] << 8) | data[2 * c + 1]);
            }
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            done = true;
        } else if (!(type[0] & 0x20)) {
            fail("unknown critical PNG chunk");
        }
        at += size_t(len) + 12;
    }
    if (!have_hdr || idat.empty()) fail("PNG without IHDR or IDAT");
    if (I.ctype == 3 && I.palette.empty()) fail("palette PNG without PLTE");
    const size_t bits_pp = size_t(I.depth) * size_t(I.channels);
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    // Adam7 pass origins and steps (PNG specification, 8.2)
    static const int px0[7] = {0, 4, 0, 2, 0, 1, 0}, py0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int dx[7] = {8, 8, 4, 4, 2, 2, 1}, dy[7] = {8, 8, 8, 4, 4, 2, 2};
    struct Pass {
        uint32_t w, h, ox, oy, sx, sy;
    };
    std::vector<Pass> passes;
    if (interlace) {
        for (int k = 0; k < 7; ++k) {
            const uint32_t w = I.w > uint32_t(px0[k]) ? (I.w - px0[k] + dx[k] - 1) / dx[k] : 0;
            const uint32_t h = I.h > uint32_t(py0[k]) ? (I.h - py0[k] + dy[k] - 1) / dy[k] : 0;
            passes.push_back({w, h, uint32_t(px0[k]), uint32_t(py0[k]), uint32_t(dx[k]), uint32_t(dy[k])});
        }
    } else {
        passes.push_back({I.w, I.h, 0, 0, 1, 1});
    }
    size_t total = 0;
    for (const Pass& ps : passes)
        if (ps.w && ps.h) total += size_t(ps.h) * ((size_t(ps.w) * bits_pp + 7) / 8 + 1);
    std::vector<uint8_t> raw = zlib_inflate(idat.data(), idat.size(), total);
    if (raw.size() != total) fail("PNG image data is truncated");
    img.width = I.w;
    img.height = I.h;
    img.rgba.assign(size_t(I.w) * I.h * 4, 0);
    size_t off = 0;
    for (const Pass& ps : passes) {
        if (!ps.w || !ps.h) continue;
        const size_t stride = (size_t(ps.w) * bits_pp + 7) / 8;
        unfilter(raw.data() + off, ps.h, stride, bpp);
        for (uint32_t y = 0; y < ps.h; ++y) {
            const uint8_t* row = raw.data() + off + size_t(y) * (stride + 1) + 1;
            uint8_t* out_row = &img.rgba[size_t(ps.oy + y * ps.sy) * I.w * 4];
            if (I.depth == 8 && I.ctype == 6 && ps.sx == 1) {  // RGBA8 rows as they are
                std::memcpy(out_row, row, size_t(ps.w) * 4);
            } else if (I.depth == 8 && I.ctype == 2 && !I.has_key) {
                for (uint32_t x = 0; x < ps.w; ++x) {
                    uint8_t* d = out_row + size_t(ps.ox + x * ps.sx) * 4;
                    d[0] = row[3 * x], d[1] = row[3 * x + 1], d[2] = row[3 * x + 2], d[3] = 255;
                }
            } else {
                for (uint32_t x = 0; x < ps.w; ++x) put_pixel(I, row, x, out_row + size_t(ps.ox + x * ps.sx) * 4);
            }
        }
        off += size_t(ps.h) * (stride + 1);
    }
}

void put_error(char* error, uint32_t cap, const char* m) {
    if (!error || !cap) return;
    std::strncpy(error, m, cap - 1);
    error[cap - 1] = '\0';
}

uint32_t le32(const uint8_t* p) {
    return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

}  // namespace

extern "C" int vkgv_image_decode_png(const void* data, uint64_t size, vkgv_image** out, char* error,
                                     uint32_t error_capacity) {
    if (!data || !out) return VKGV_INVALID_ARG;
    *out = nullptr;
    vkgv_image* img = new (std::nothrow) vkgv_image();
    if (!img) return VKGV_OUT_OF_MEMORY;
    try {
        decode_png(static_cast<const uint8_t*>(data), size_t(size), *img);
    } catch (const DecodeError& e) {
        put_error(error, error_capacity, e.msg);
        delete img;
        return VKGV_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        put_error(error, error_capacity, "out of host memory");
        delete img;
        return VKGV_OUT_OF_MEMORY;
    }
    *out = img;
    return VKGV_OK;
}

extern "C" int vkgv_image_get(const vkgv_image* img, uint32_t* width, uint32_t* height, const uint8_t** rgba) {
    if (!img) return VKGV_INVALID_ARG;
    if (width) *width = img->width;
    if (height) *height = img->height;
    if (rgba) *rgba = img->rgba.data();
    return VKGV_OK;
}

extern "C" void vkgv_image_free(vkgv_image* img) { delete img; }

// DDS: "DDS " + DDS_HEADER (124 B) [+ DDS_HEADER_DXT10 (20 B)], top mip first.
extern "C" int vkgv_dds_parse(const void* data, uint64_t size, vkgv_dds_info* out) {
    if (!data || !out) return VKGV_INVALID_ARG;
    const uint8_t* p = static_cast<const uint8_t*>(data);
    std::memset(out, 0, sizeof(*out));
    if (size < 128 || std::memcmp(p, "DDS ", 4) != 0 || le32(p + 4) != 124) return VKGV_INVALID_ARG;
    out->height = le32(p + 12);
    out->width = le32(p + 16);
    out->mip_count = std::max<uint32_t>(1, le32(p + 28));
    // far beyond any texture edge the decoders accept; keeps the byte counts
    // below 2^64
    if (out->width > (1u << 20) || out->height > (1u << 20)) return VKGV_INVALID_ARG;
    const uint32_t pf_flags = le32(p + 80), fourcc = le32(p + 84);
    uint64_t offset = 128;
    uint32_t fmt = 0;
    auto finish = [&](uint32_t format, uint64_t bytes) {
        out->format = format;
        out->data_offset = offset;
        out->data_size = bytes;
        if (out->width == 0 || out->height == 0 || offset + bytes > size) return VKGV_INVALID_ARG;
        return VKGV_OK;
    };
    const uint64_t texels = uint64_t(out->width) * out->height;
    if (!(pf_flags & 0x4)) {
        // DDPF_RGB (0x40): 32-bit texels whose channel masks are RGBA or
        // BGRA bytes (DDPF_ALPHAPIXELS 0x1 says the top byte is alpha;
        // without it the texels are opaque and read as alpha 255)
        const uint32_t bits = le32(p + 88), rm = le32(p + 92), gm = le32(p + 96), bm = le32(p + 100);
        if (!(pf_flags & 0x40) || bits != 32 || gm != 0x0000FF00u) return VKGV_INVALID_ARG;
        const bool alpha = (pf_flags & 0x1) != 0;
        if (rm == 0x000000FFu && bm == 0x00FF0000u) fmt = alpha ? VKGV_RGBA8 : VKGV_RGBX8;
        else if (rm == 0x00FF0000u && bm == 0x000000FFu) fmt = alpha ? VKGV_BGRA8 : VKGV_BGRX8;
        else return VKGV_INVALID_ARG;
        return finish(fmt, texels * 4);
    }
    auto cc = [](const char* s) { return uint32_t(s[0]) | (uint32_t(s[1]) << 8) | (uint32_t(s[2]) << 16) | (uint32_t(s[3]) << 24); };
    if (fourcc == cc("DXT1")) fmt = VKGV_BC1;
    else if (fourcc == cc("DXT2") || fourcc == cc("DXT3")) fmt = VKGV_BC2;
    else if (fourcc == cc("DXT4") || fourcc == cc("DXT5")) fmt = VKGV_BC3;
    else if (fourcc == cc("ATI1") || fourcc == cc("BC4U")) fmt = VKGV_BC4;
    else if (fourcc == cc("ATI2") || fourcc == cc("BC5U")) fmt = VKGV_BC5;
    else if (fourcc == cc("DX10")) {
        if (size < 148) return VKGV_INVALID_ARG;
        const uint32_t dxgi = le32(p + 128);
        offset = 148;
        switch (dxgi) {  // DXGI_FORMAT_BC*_UNORM and *_UNORM_SRGB
            case 28: case 29: return (out->srgb = dxgi == 29, finish(VKGV_RGBA8, texels * 4));  // R8G8B8A8_UNORM(_SRGB)
            case 87: case 91: return (out->srgb = dxgi == 91, finish(VKGV_BGRA8, texels * 4));  // B8G8R8A8_UNORM(_SRGB)
            case 88: case 93: return (out->srgb = dxgi == 93, finish(VKGV_BGRX8, texels * 4));  // B8G8R8X8_UNORM(_SRGB)
            case 71: case 72: fmt = VKGV_BC1; break;
            case 74: case 75: fmt = VKGV_BC2; break;
            case 77: case 78: fmt = VKGV_BC3; break;
            case 80: fmt = VKGV_BC4; break;
            case 83: fmt = VKGV_BC5; break;
            case 98: case 99: fmt = VKGV_BC7; break;  // DXGI_FORMAT_BC7_UNORM(_SRGB)
            case 95: fmt = VKGV_BC6H_UF16; break;     // DXGI_FORMAT_BC6H_UF16
            case 96: fmt = VKGV_BC6H_SF16; break;     // DXGI_FORMAT_BC6H_SF16
            default: return VKGV_INVALID_ARG;
        }
        out->srgb = (dxgi == 72 || dxgi == 75 || dxgi == 78 || dxgi == 99) ? 1u : 0u;
    } else {
        return VKGV_INVALID_ARG;
    }
    out->format = fmt;
    out->data_offset = offset;
    const uint64_t bw = (uint64_t(out->width) + 3) / 4, bh = (uint64_t(out->height) + 3) / 4;
    out->data_size = bw * bh * ((fmt == VKGV_BC1 || fmt == VKGV_BC4) ? 8u : 16u);
    if (out->width == 0 || out->height == 0 || offset + out->data_size > size) return VKGV_INVALID_ARG;
    return VKGV_OK;
}

// KTX 2.0: the 12-byte identifier, nine uint32 header words (vkFormat,
// typeSize, pixelWidth, pixelHeight, pixelDepth, layerCount, faceCount,
// levelCount, supercompressionScheme), the index (DFD and KVD offsets and
// lengths as uint32, SGD as uint64) and one {byteOffset, byteLength,
// uncompressedByteLength} uint64 triple per level, level 0 the largest.
extern "C" int vkgv_ktx2_parse(const void* data, uint64_t size, vkgv_dds_info* out) {
    static const uint8_t kId[12] = {0xAB, 'K', 'T', 'X', ' ', '2', '0', 0xBB, '\r', '\n', 0x1A, '\n'};
    if (!data || !out) return VKGV_INVALID_ARG;
    const uint8_t* p = static_cast<const uint8_t*>(data);
    std::memset(out, 0, sizeof(*out));
    if (size < 80 + 24 || std::memcmp(p, kId, 12) != 0) return VKGV_INVALID_ARG;
    const uint32_t vk_format = le32(p + 12), width = le32(p + 20), height = le32(p + 24);
    const uint32_t depth = le32(p + 28), layers = le32(p + 32), faces = le32(p + 36);
    const uint32_t levels = le32(p + 40), scheme = le32(p + 44);
    if ((scheme != 0 && scheme != 2) || vk_format == 0) return VKGV_INVALID_ARG;  // BasisU / BasisLZ
    if (width == 0 || height == 0 || depth > 1 || layers > 1 || faces != 1) return VKGV_INVALID_ARG;
    if (width > (1u << 20) || height > (1u << 20)) return VKGV_INVALID_ARG;  // byte counts stay below 2^64
    uint32_t fmt = 0, srgb = 0;
    switch (vk_format) {  // VkFormat values
        case 131: fmt = VKGV_BC1_OPAQUE; break;           // BC1_RGB_UNORM_BLOCK
        case 132: fmt = VKGV_BC1_OPAQUE; srgb = 1; break;  // BC1_RGB_SRGB_BLOCK
        case 133: fmt = VKGV_BC1; break;
        case 134: fmt = VKGV_BC1; srgb = 1; break;
        case 135: fmt = VKGV_BC2; break;
        case 136: fmt = VKGV_BC2; srgb = 1; break;
        case 137: fmt = VKGV_BC3; break;
        case 138: fmt = VKGV_BC3; srgb = 1; break;
        case 139: fmt = VKGV_BC4; break;                   // BC4_UNORM_BLOCK
        case 141: fmt = VKGV_BC5; break;                   // BC5_UNORM_BLOCK
        case 145: fmt = VKGV_BC7; break;                   // BC7_UNORM_BLOCK
        case 146: fmt = VKGV_BC7; srgb = 1; break;         // BC7_SRGB_BLOCK
        case 143: fmt = VKGV_BC6H_UF16; break;             // BC6H_UFLOAT_BLOCK
        case 144: fmt = VKGV_BC6H_SF16; break;             // BC6H_SFLOAT_BLOCK
        case 37: fmt = VKGV_RGBA8; break;                  // R8G8B8A8_UNORM
        case 43: fmt = VKGV_RGBA8; srgb = 1; break;        // R8G8B8A8_SRGB
        default: return VKGV_INVALID_ARG;
    }
    uint64_t offset, length, raw_length;
    std::memcpy(&offset, p + 80, 8);
    std::memcpy(&length, p + 88, 8);
    std::memcpy(&raw_length, p + 96, 8);
    uint64_t need;
    if (fmt == VKGV_RGBA8) {
        need = uint64_t(width) * height * 4;
    } else {
        const uint64_t bw = (uint64_t(width) + 3) / 4, bh = (uint64_t(height) + 3) / 4;
        need = bw * bh * ((fmt == VKGV_BC1 || fmt == VKGV_BC4 || fmt == VKGV_BC1_OPAQUE) ? 8u : 16u);
    }
    if (scheme == 2) {
        // a zstd level: its compressed bytes in the file, the texels after
        // inflating
        if (raw_length != need || length == 0 || offset > size || size - offset < length) return VKGV_INVALID_ARG;
    } else if (length < need || offset > size || size - offset < need) {
        return VKGV_INVALID_ARG;
    }
    out->width = width;
    out->height = height;
    out->mip_count = levels ? levels : 1;
    out->format = fmt;
    out->srgb = srgb;
    out->supercompression = scheme;
    out->data_offset = offset;
    out->data_size = scheme == 2 ? length : need;
    return VKGV_OK;
}
