// EXT_meshopt_compression buffer views: the work of the reference's
// MeshoptDecompressor::ExecuteRange (src/vk_gltf_viewer/assets.cpp:111-166),
// which calls meshoptimizer's vertex, index and index-sequence decoders and
// its octahedral / quaternion / exponential filters on every compressed
// bufferView.  meshoptimizer is an empty submodule in the reference (no
// pinned commit), so this restates the bitstreams of the published
// EXT_meshopt_compression specification:
//
//   ATTRIBUTES (header 0xA0): vertices in blocks of
//     min(8192 / stride rounded down to 16, 256); per block, per byte
//     position of the vertex, a column of byte deltas (zig-zag, against the
//     previous vertex, the first block against the baseline vertex stored in
//     the last `stride` bytes of the stream) in groups of 16, each group
//     0 = all zero, 1 = 2-bit codes, 2 = 4-bit codes (the all-ones code
//     escapes to a literal byte after the group's codes), 3 = 16 literal bytes,
//     the 2-bit group modes packed four per header byte, low bits first, the
//     codes most significant bits first; a tail of max(32, stride) bytes.
//   TRIANGLES (header 0xE0 | version, version 0 or 1): one code byte per
//     triangle, then variable-length data, then a 16-byte table of auxiliary
//     codes; a 16-entry edge FIFO, a 16-entry vertex FIFO, the next new index
//     and the last explicit index rebuild each triangle (below).
//   INDICES (header 0xD0 | version): one varint per index, its low bit
//     selecting one of two running baselines, the rest a zig-zag delta; a
//     4-byte tail.
//   Filters, in place after ATTRIBUTES decoding: OCTAHEDRAL (4 x int8 or
//     4 x int16: x, y on the octahedron, z = the encoded 1.0, w kept),
//     QUATERNION (4 x int16: three components, the fourth holding the scale
//     and the index of the dropped largest component), EXPONENTIAL
//     (int32: 24-bit signed mantissa, 8-bit signed exponent).
//
// The filters' float arithmetic is pinned (plain IEEE fp32 operations in
// the order written, no fused multiply-add, round half away from zero);
// the oracle restates the same operations.  Unlike the reference, which
// ignores the decoders' status (assets.cpp:146-147) and keeps whatever was
// written, a stream that does not decode to exactly its declared length is
// an error.  Host code, run once per asset.
#include "vkgv.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint8_t unzigzag8(uint8_t v) { return uint8_t((v >> 1) ^ uint8_t(0u - (v & 1u))); }
inline uint32_t unzigzag32(uint32_t v) { return (v >> 1) ^ (0u - (v & 1u)); }

// Little-endian base-128 varint of at most five bytes.
inline uint32_t read_varint(const uint8_t*& p) {
    uint32_t v = 0;
    for (int i = 0; i < 5; ++i) {
        const uint8_t b = *p++;
        v |= uint32_t(b & 127u) << (7 * i);
        if (b < 128) break;
    }
    return v;
}

inline void put_index(uint8_t* dst, size_t stride, size_t i, uint32_t v) {
    if (stride == 2) {
        const uint16_t s = uint16_t(v);
        std::memcpy(dst + 2 * i, &s, 2);
    } else {
        std::memcpy(dst + 4 * i, &v, 4);
    }
}

// ------------------------------------------------------------ attributes

// A group of 16 byte deltas needs at most 24 bytes (8 of 4-bit codes and 16
// escapes); the stream's tail guarantees that much room before each group.
constexpr size_t kGroupRoom = 24;

// One column of `groups * 16` byte deltas; nullptr if the stream runs out.
const uint8_t* read_column(const uint8_t* p, const uint8_t* end, size_t groups, uint8_t* out) {
    const size_t header_bytes = (groups + 3) / 4;
    if (size_t(end - p) < header_bytes) return nullptr;
    const uint8_t* modes = p;
    p += header_bytes;
    for (size_t g = 0; g < groups; ++g) {
        if (size_t(end - p) < kGroupRoom) return nullptr;
        const unsigned mode = (modes[g / 4] >> (2 * (g % 4))) & 3u;
        uint8_t* o = out + 16 * g;
        if (mode == 0) {
            std::memset(o, 0, 16);
        } else if (mode == 3) {
            std::memcpy(o, p, 16);
            p += 16;
        } else if (mode == 1) {
            // 16 two-bit codes, the first in the top bits; code 3 escapes
            const uint32_t w = uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3];
            const uint8_t* literal = p + 4;
            if ((w & (w >> 1) & 0x55555555u) == 0) {
                for (unsigned i = 0; i < 16; ++i) o[i] = uint8_t((w >> (30 - 2 * i)) & 3u);
            } else {
                for (unsigned i = 0; i < 16; ++i) {
                    const unsigned code = (w >> (30 - 2 * i)) & 3u;
                    o[i] = code == 3u ? *literal++ : uint8_t(code);
                }
            }
            p = literal;
        } else {
            // 16 four-bit codes; code 15 escapes
            uint64_t w = 0;
            for (int i = 0; i < 8; ++i) w = w << 8 | p[i];
            const uint8_t* literal = p + 8;
            if ((w & (w >> 1) & (w >> 2) & (w >> 3) & 0x1111111111111111ull) == 0) {
                for (unsigned i = 0; i < 16; ++i) o[i] = uint8_t((w >> (60 - 4 * i)) & 15u);
            } else {
                for (unsigned i = 0; i < 16; ++i) {
                    const unsigned code = unsigned(w >> (60 - 4 * i)) & 15u;
                    o[i] = code == 15u ? *literal++ : uint8_t(code);
                }
            }
            p = literal;
        }
    }
    return p;
}

// The stream length of one group of mode 1 or 2 from its codes: the codes
// plus one byte per escape.
inline size_t group_length(unsigned mode, const uint8_t* p) {
    if (mode == 0) return 0;
    if (mode == 3) return 16;
    if (mode == 1) {
        const uint32_t w = uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3];
        return 4 + size_t(__builtin_popcount(w & (w >> 1) & 0x55555555u));
    }
    uint64_t w = 0;
    for (int i = 0; i < 8; ++i) w = w << 8 | p[i];
    return 8 + size_t(__builtin_popcountll(w & (w >> 1) & (w >> 2) & (w >> 3) & 0x1111111111111111ull));
}

// Where each block's data starts, by walking the group lengths without
// decoding; fails exactly where read_column would.  Returns the end of the
// last block.
const uint8_t* scan_blocks(const uint8_t* p, const uint8_t* end, size_t count, size_t stride, size_t block,
                           std::vector<const uint8_t*>& starts) {
    for (size_t first = 0; first < count; first += block) {
        starts.push_back(p);
        const size_t groups = (std::min(block, count - first) + 15) / 16;
        for (size_t k = 0; k < stride; ++k) {
            const size_t header_bytes = (groups + 3) / 4;
            if (size_t(end - p) < header_bytes) return nullptr;
            const uint8_t* modes = p;
            p += header_bytes;
            for (size_t g = 0; g < groups; ++g) {
                if (size_t(end - p) < kGroupRoom) return nullptr;
                p += group_length((modes[g / 4] >> (2 * (g % 4))) & 3u, p);
            }
        }
    }
    return p;
}

// Blocks [b0, b1) from their stream starts, the chain of each byte column
// starting at prev.
bool decode_blocks(uint8_t* dst, size_t count, size_t stride, size_t block, const uint8_t* const* starts,
                   const uint8_t* end, size_t b0, size_t b1, uint8_t prev[256]) {
    uint8_t deltas[256];
    for (size_t b = b0; b < b1; ++b) {
        const uint8_t* p = starts[b];
        const size_t first = b * block, n = std::min(block, count - first);
        for (size_t k = 0; k < stride; ++k) {
            p = read_column(p, end, (n + 15) / 16, deltas);
            if (!p) return false;
            uint8_t v = prev[k];
            uint8_t* out = dst + first * stride + k;
            for (size_t i = 0; i < n; ++i) {
                v = uint8_t(v + unzigzag8(deltas[i]));
                out[i * stride] = v;
            }
            prev[k] = v;
        }
    }
    return true;
}

// Views of at least this many decoded bytes split their blocks over threads.
constexpr size_t kThreadedBytes = size_t(4) << 20;

bool decode_attributes(uint8_t* dst, size_t count, size_t stride, const uint8_t* src, size_t size, unsigned threads) {
    if (stride == 0 || stride > 256 || stride % 4 != 0) return false;
    if (size < 1 + stride || src[0] != 0xA0) return false;
    const uint8_t* end = src + size;
    uint8_t prev[256];
    std::memcpy(prev, end - stride, stride);
    const size_t block = std::min<size_t>((8192 / stride) & ~size_t(15), 256);
    const size_t blocks = (count + block - 1) / block;
    std::vector<const uint8_t*> starts;
    starts.reserve(blocks);
    const uint8_t* tail = scan_blocks(src + 1, end, count, stride, block, starts);
    if (!tail || size_t(end - tail) != std::max<size_t>(stride, 32)) return false;
    threads = unsigned(std::min<size_t>({size_t(threads), blocks, count * stride / (kThreadedBytes / 4) + 1}));
    if (threads <= 1 || count * stride < kThreadedBytes) return decode_blocks(dst, count, stride, block, starts.data(), end, 0, blocks, prev);
    // chunks of blocks decode at once, each chain starting from zero (chunk
    // 0 from the baseline); byte deltas add mod 256, so every later chunk
    // then takes the true last vertex of the chunk before it as a carry
    std::vector<std::array<uint8_t, 256>> last(threads);
    std::vector<size_t> bounds(threads + 1);
    for (unsigned t = 0; t <= threads; ++t) bounds[t] = blocks * t / threads;
    std::vector<char> ok(threads, 0);
    {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < threads; ++t)
            pool.emplace_back([&, t] {
                if (t == 0) std::memcpy(last[0].data(), prev, stride);
                else std::memset(last[t].data(), 0, stride);
                ok[t] = decode_blocks(dst, count, stride, block, starts.data(), end, bounds[t], bounds[t + 1],
                                      last[t].data());
            });
        for (auto& th : pool) th.join();
    }
    for (unsigned t = 0; t < threads; ++t)
        if (!ok[t]) return false;
    std::vector<std::array<uint8_t, 256>> carry(threads);
    for (unsigned t = 1; t < threads; ++t)
        for (size_t k = 0; k < stride; ++k) {
            carry[t][k] = last[t - 1][k];
            last[t][k] = uint8_t(last[t][k] + carry[t][k]);
        }
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t)
        pool.emplace_back([&, t] {
            const size_t v0 = bounds[t] * block, v1 = std::min(count, bounds[t + 1] * block);
            uint8_t row[256];
            std::memcpy(row, carry[t].data(), stride);
            for (size_t v = v0; v < v1; ++v) {
                uint8_t* out = dst + v * stride;
                for (size_t k = 0; k < stride; ++k) out[k] = uint8_t(out[k] + row[k]);
            }
        });
    for (auto& th : pool) th.join();
    return true;
}

// ------------------------------------------------------------- triangles

struct TriangleFifos {
    uint32_t edge[16][2];
    uint32_t vert[16];
    unsigned edge_head = 0, vert_head = 0;  // next slot to write
    uint32_t next = 0, last = 0;            // next new index, last explicit index

    TriangleFifos() {
        std::memset(edge, 0xFF, sizeof(edge));
        std::memset(vert, 0xFF, sizeof(vert));
    }
    // k-th most recent edge (k = 0: the newest)
    const uint32_t* edge_at(unsigned k) const { return edge[(edge_head - 1 - k) & 15u]; }
    // the vertex k places back from the write slot (k = 1: the newest)
    uint32_t vert_back(unsigned k) const { return vert[(vert_head - k) & 15u]; }
    void push_edge(uint32_t a, uint32_t b) {
        edge[edge_head][0] = a;
        edge[edge_head][1] = b;
        edge_head = (edge_head + 1) & 15u;
    }
    void push_vert(uint32_t v) {
        vert[vert_head] = v;
        vert_head = (vert_head + 1) & 15u;
    }
    uint32_t explicit_index(const uint8_t*& p) { return last = last + unzigzag32(read_varint(p)); }
};

bool decode_triangles(uint8_t* dst, size_t count, size_t stride, const uint8_t* src, size_t size) {
    if ((stride != 2 && stride != 4) || count % 3 != 0) return false;
    const size_t tris = count / 3;
    if (size < 1 + tris + 16 || (src[0] & 0xF0) != 0xE0 || (src[0] & 15) > 1) return false;
    // third-vertex codes from `explicit_from` up are explicit indices
    // (version 1: 13 = last - 1, 14 = last + 1, 15 = a varint delta)
    const unsigned explicit_from = (src[0] & 15) ? 13 : 15;
    const uint8_t* codes = src + 1;
    const uint8_t* p = codes + tris;
    const uint8_t* data_end = src + size - 16;  // the auxiliary-code table follows
    const uint8_t* table = data_end;
    TriangleFifos F;
    for (size_t t = 0; t < tris; ++t) {
        if (p > data_end) return false;  // a triangle reads at most 16 bytes, the table's size
        const uint8_t code = codes[t];
        uint32_t a, b, c;
        if (code < 0xF0) {
            // an edge of a recent triangle, and a third vertex
            const uint32_t* e = F.edge_at(code >> 4);
            a = e[0];
            b = e[1];
            const unsigned fc = code & 15u;
            if (fc == 0) {
                c = F.next++;
                F.push_vert(c);
            } else if (fc < explicit_from) {
                c = F.vert[(F.vert_head - 1 - fc) & 15u];  // a recent vertex, not pushed again
            } else {
                c = fc == 15 ? F.explicit_index(p) : (F.last = F.last + (fc == 13 ? 0xFFFFFFFFu : 1u));
                F.push_vert(c);
            }
            F.push_edge(c, b);
            F.push_edge(a, c);
        } else {
            // a triangle sharing no recent edge: a is new (or explicit),
            // b and c are new, recent or explicit
            const bool table_code = code < 0xFE;
            const uint8_t aux = table_code ? table[code & 15u] : *p++;
            const unsigned fb = aux >> 4, fc = aux & 15u;
            if (!table_code && aux == 0) F.next = 0;  // restart the new-index counter
            a = code == 0xFF ? 0u : F.next++;
            b = fb == 0 ? F.next++ : F.vert_back(fb);
            c = fc == 0 ? F.next++ : F.vert_back(fc);
            if (!table_code) {
                if (code == 0xFF) a = F.explicit_index(p);
                if (fb == 15) b = F.explicit_index(p);
                if (fc == 15) c = F.explicit_index(p);
            }
            F.push_vert(a);
            if (fb == 0 || (!table_code && fb == 15)) F.push_vert(b);
            if (fc == 0 || (!table_code && fc == 15)) F.push_vert(c);
            F.push_edge(b, a);
            F.push_edge(c, b);
            F.push_edge(a, c);
        }
        put_index(dst, stride, 3 * t + 0, a);
        put_index(dst, stride, 3 * t + 1, b);
        put_index(dst, stride, 3 * t + 2, c);
    }
    return p == data_end;
}

// --------------------------------------------------------- index sequence

bool decode_sequence(uint8_t* dst, size_t count, size_t stride, const uint8_t* src, size_t size) {
    if (stride != 2 && stride != 4) return false;
    if (size < 1 + count + 4 || (src[0] & 0xF0) != 0xD0 || (src[0] & 15) > 1) return false;
    const uint8_t* p = src + 1;
    const uint8_t* data_end = src + size - 4;
    uint32_t base[2] = {0, 0};
    for (size_t i = 0; i < count; ++i) {
        if (p >= data_end) return false;  // a varint reads at most 5 bytes
        const uint32_t v = read_varint(p);
        uint32_t& b = base[v & 1u];
        b += unzigzag32(v >> 1);
        put_index(dst, stride, i, b);
    }
    return p == data_end;
}

// --------------------------------------------------------------- filters

inline float round_away(float v) { return v >= 0.0f ? v + 0.5f : v - 0.5f; }

template <class T>
void filter_octahedral(uint8_t* data, size_t count) {
    const float one = float((1 << (8 * sizeof(T) - 1)) - 1);
    for (size_t i = 0; i < count; ++i) {
        T q[4];
        std::memcpy(q, data + i * sizeof(q), sizeof(q));
        float x = float(q[0]), y = float(q[1]);
        const float z = float(q[2]) - std::fabs(x) - std::fabs(y);
        const float fold = std::min(z, 0.0f);  // the lower hemisphere folds over the diagonals
        x += x >= 0.0f ? fold : -fold;
        y += y >= 0.0f ? fold : -fold;
        const float len = std::sqrt(x * x + y * y + z * z);
        if (len == 0.0f) {
            q[0] = q[1] = q[2] = 0;
        } else {
            const float s = one / len;
            q[0] = T(int32_t(round_away(x * s)));
            q[1] = T(int32_t(round_away(y * s)));
            q[2] = T(int32_t(round_away(z * s)));
        }
        std::memcpy(data + i * sizeof(q), q, sizeof(q));
    }
}

void filter_quaternion(uint8_t* data, size_t count) {
    const float inv_sqrt2 = 1.0f / std::sqrt(2.0f);
    for (size_t i = 0; i < count; ++i) {
        int16_t q[4];
        std::memcpy(q, data + 8 * i, 8);
        const float s = inv_sqrt2 / float(int32_t(q[3]) | 3);
        const float x = float(q[0]) * s, y = float(q[1]) * s, z = float(q[2]) * s;
        const float ww = 1.0f - x * x - y * y - z * z;
        const float w = std::sqrt(std::max(ww, 0.0f));
        const unsigned largest = unsigned(q[3]) & 3u;
        int16_t out[4];
        out[(largest + 1) & 3u] = int16_t(uint16_t(int32_t(round_away(x * 32767.0f))));
        out[(largest + 2) & 3u] = int16_t(uint16_t(int32_t(round_away(y * 32767.0f))));
        out[(largest + 3) & 3u] = int16_t(uint16_t(int32_t(round_away(z * 32767.0f))));
        out[largest] = int16_t(uint16_t(int32_t(w * 32767.0f + 0.5f)));
        std::memcpy(data + 8 * i, out, 8);
    }
}

void filter_exponential(uint8_t* data, size_t words) {
    for (size_t i = 0; i < words; ++i) {
        uint32_t v;
        std::memcpy(&v, data + 4 * i, 4);
        const int32_t mantissa = int32_t(v << 8) >> 8, exponent = int32_t(v) >> 24;
        const float f = std::ldexp(float(mantissa), exponent);
        std::memcpy(data + 4 * i, &f, 4);
    }
}

}  // namespace

namespace vkgv {

// Views of fewer bytes than this decode on one thread; larger ATTRIBUTES
// views split their blocks over up to `threads`.
size_t meshopt_threaded_bytes() { return kThreadedBytes; }

int meshopt_decode(void* dst, uint64_t count, uint64_t stride, const void* src, uint64_t size, int mode, int filter,
                   unsigned threads) {
    if (!dst || (!src && size) || stride == 0 || count > (uint64_t(1) << 40) / stride) return VKGV_INVALID_ARG;
    if (filter != VKGV_MESHOPT_FILTER_NONE && mode != VKGV_MESHOPT_ATTRIBUTES) return VKGV_INVALID_ARG;
    if (filter == VKGV_MESHOPT_FILTER_OCTAHEDRAL && stride != 4 && stride != 8) return VKGV_INVALID_ARG;
    if (filter == VKGV_MESHOPT_FILTER_QUATERNION && stride != 8) return VKGV_INVALID_ARG;
    if (filter < VKGV_MESHOPT_FILTER_NONE || filter > VKGV_MESHOPT_FILTER_EXPONENTIAL) return VKGV_INVALID_ARG;
    auto* out = static_cast<uint8_t*>(dst);
    const auto* in = static_cast<const uint8_t*>(src);
    bool ok = false;
    switch (mode) {
    case VKGV_MESHOPT_ATTRIBUTES: ok = decode_attributes(out, count, stride, in, size, threads); break;
    case VKGV_MESHOPT_TRIANGLES: ok = decode_triangles(out, count, stride, in, size); break;
    case VKGV_MESHOPT_INDICES: ok = decode_sequence(out, count, stride, in, size); break;
    default: return VKGV_INVALID_ARG;
    }
    if (!ok) return VKGV_INVALID_ARG;
    switch (filter) {
    case VKGV_MESHOPT_FILTER_OCTAHEDRAL:
        if (stride == 4) filter_octahedral<int8_t>(out, count);
        else filter_octahedral<int16_t>(out, count);
        break;
    case VKGV_MESHOPT_FILTER_QUATERNION: filter_quaternion(out, count); break;
    case VKGV_MESHOPT_FILTER_EXPONENTIAL: filter_exponential(out, count * stride / 4); break;
    default: break;
    }
    return VKGV_OK;
}

}  // namespace vkgv

extern "C" int vkgv_meshopt_decode(void* dst, uint64_t count, uint64_t stride, const void* src, uint64_t size,
                                   int mode, int filter) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    try {
        return vkgv::meshopt_decode(dst, count, stride, src, size, mode, filter, std::min(hw, 16u));
    } catch (...) {  // thread or scratch creation
        return VKGV_OUT_OF_MEMORY;
    }
}
