// Block-compressed texture decode on the device: BC1-BC5 (the DXT1-5 /
// RGTC formats a DDS base-colour texture holds, MSFT_texture_dds) and BC7 into RGBA8
// for the textured resolve, and BC6H into float32 RGB.  The reference loads no images
// (src/vk_gltf_viewer/assets.cpp:467-471); the formats are the published
// ones, with the interpolation rounding, which they leave to the
// implementation, pinned here and in the oracle:
//   RGB565 -> 8 bits: (r5 << 3 | r5 >> 2), (g6 << 2 | g6 >> 4)
//   BC1 (c0 > c1) and BC2/BC3 colours: c2 = (2 c0 + c1 + 1) / 3,
//                                      c3 = (c0 + 2 c1 + 1) / 3
//   BC1 (c0 <= c1): c2 = (c0 + c1 + 1) / 2, c3 = transparent black (opaque
//     black for VKGV_BC1_OPAQUE, Vulkan's BC1_RGB formats)
//   BC2 alpha: a4 * 17
//   BC3 alpha / BC4 / BC5 channels (a0 > a1): a_i = ((7 - i) a0 + i a1 + 3) / 7
//     for the interpolated codes i = 1..6 (indices 2..7);
//     (a0 <= a1): a_i = ((5 - i) a0 + i a1 + 2) / 5 for i = 1..4 (indices 2..5),
//     index 6 = 0, index 7 = 255
//   BC4 -> (r, 0, 0, 255), BC5 -> (r, g, 0, 255)
// One thread per block row: the four rows of a block share its load and
// each writes 4 texels, so a warp stores four contiguous 128-byte rows.
#include <cuda_fp16.h>

#include "kernels.cuh"

namespace vkgv {

namespace {

constexpr int kDecodeWarps = 8;  // warps per CTA; a warp decodes 8 blocks x 4 rows per block row
constexpr int kDecodeDepth = 4;  // block rows of y per thread

__device__ __forceinline__ uint32_t rgb565(uint32_t c) {
    const uint32_t r = (c >> 11) & 31u, g = (c >> 5) & 63u, b = c & 31u;
    return ((r << 3) | (r >> 2)) | (((g << 2) | (g >> 4)) << 8) | (((b << 3) | (b >> 2)) << 16);
}

__device__ __forceinline__ uint32_t ch(uint32_t c, int k) { return (c >> (8 * k)) & 255u; }

// The four RGBA entries of a BC1-layout colour block (words lo = c0 | c1 << 16).
__device__ __forceinline__ void colour_palette(uint32_t lo, bool allow_three, bool opaque, uint32_t pal[4]) {
    const uint32_t c0 = lo & 0xFFFFu, c1 = lo >> 16;
    const uint32_t a = rgb565(c0), b = rgb565(c1);
    const bool four = !allow_three || c0 > c1;
    uint32_t p2 = 0, p3 = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t x = ch(a, k), y = ch(b, k);
        p2 |= (four ? (2 * x + y + 1) / 3 : (x + y + 1) / 2) << (8 * k);
        p3 |= (four ? (x + 2 * y + 1) / 3 : 0u) << (8 * k);
    }
    pal[0] = a | 0xFF000000u;
    pal[1] = b | 0xFF000000u;
    pal[2] = p2 | 0xFF000000u;
    pal[3] = four ? (p3 | 0xFF000000u) : (opaque ? 0xFF000000u : 0u);
}

// The 4 values of row r of an interpolated channel block (8 bytes, as lo/hi
// words): its 8-entry palette packed as bytes into two words, then one byte
// per texel.
__device__ __forceinline__ void channel_row(uint32_t lo, uint32_t hi, uint32_t r, uint32_t out[4]) {
    const uint32_t a0 = lo & 255u, a1 = (lo >> 8) & 255u;
    uint32_t v[8];
    v[0] = a0;
    v[1] = a1;
    if (a0 > a1) {
#pragma unroll
        for (uint32_t j = 1; j <= 6; ++j) v[j + 1] = ((7 - j) * a0 + j * a1 + 3) / 7;
    } else {
#pragma unroll
        for (uint32_t j = 1; j <= 4; ++j) v[j + 1] = ((5 - j) * a0 + j * a1 + 2) / 5;
        v[6] = 0;
        v[7] = 255;
    }
    const uint32_t p0 = v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
    const uint32_t p1 = v[4] | (v[5] << 8) | (v[6] << 16) | (v[7] << 24);
    const uint64_t bits = ((uint64_t)hi << 16) | (lo >> 16);  // 48 bits of 3-bit codes
    const uint32_t row = (uint32_t)(bits >> (12 * r)) & 0xFFFu;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const uint32_t c = (row >> (3 * x)) & 7u;
        out[x] = ((c < 4 ? p0 : p1) >> (8 * (c & 3u))) & 255u;
    }
}

// BC7 (BPTC UNORM), decoded as the published format defines it: the mode from the
// lowest set bit of the first byte; per mode the subset count, partition
// bits, rotation and index-selection bits, colour / alpha endpoint bits,
// p-bits (per endpoint or shared per subset) and one or two index sets;
// endpoints expanded to 8 bits by replicating their top bits; texels
// interpolated as ((64 - w) e0 + w e1 + 32) >> 6 with the 2-, 3- and 4-bit
// weight tables; the anchor texel of each subset stores one index bit less.
// A reserved mode (first byte 0) decodes to transparent black.  The
// partition and anchor tables below are the format's own.
__constant__ uint16_t c_bc7_p2[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800,
    0xFFE8, 0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE,
    0x088C, 0x3110, 0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC,
    0x3C3C, 0x55AA, 0x9696, 0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660,
    0x0272, 0x04E4, 0x4E40, 0x2720, 0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718,
    0xCCF0, 0x0FCC, 0x7744, 0xEE22};
// 3-subset partitions: two bits per texel, texel 0 in the lowest bits
__constant__ uint32_t c_bc7_p3[64] = {
    0xAA685050, 0x6A5A5040, 0x5A5A4200, 0x5450A0A8, 0xA5A50000, 0xA0A05050, 0x5555A0A0, 0x5A5A5050,
    0xAA550000, 0xAA555500, 0xAAAA5500, 0x90909090, 0x94949494, 0xA4A4A4A4, 0xA9A59450, 0x2A0A4250,
    0xA5945040, 0x0A425054, 0xA5A5A500, 0x55A0A0A0, 0xA8A85454, 0x6A6A4040, 0xA4A45000, 0x1A1A0500,
    0x0050A4A4, 0xAAA59090, 0x14696914, 0x69691400, 0xA08585A0, 0xAA821414, 0x50A4A450, 0x6A5A0200,
    0xA9A58000, 0x5090A0A8, 0xA8A09050, 0x24242424, 0x00AA5500, 0x24924924, 0x24499224, 0x50A50A50,
    0x500AA550, 0xAAAA4444, 0x66660000, 0xA5A0A5A0, 0x50A050A0, 0x69286928, 0x44AAAA44, 0x66666600,
    0xAA444444, 0x54A854A8, 0x95809580, 0x96969600, 0xA85454A8, 0x80959580, 0xAA141414, 0x96960000,
    0xAAAA1414, 0xA05050A0, 0xA0A5A5A0, 0x96000000, 0x40804080, 0xA9A8A9A8, 0xAAAAAA44, 0x2A4A5254};
__constant__ uint8_t c_bc7_a2[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8, 2, 2, 8, 8, 15, 2, 8,
    2, 2, 8, 8, 2, 2, 15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2,
    2, 15, 15, 15, 15, 15, 2, 2, 15};
__constant__ uint8_t c_bc7_a3a[64] = {
    3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5,
    15, 15, 8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5,
    10, 8, 13, 15, 12, 3, 3};
__constant__ uint8_t c_bc7_a3b[64] = {
    15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6,
    10, 15, 15, 10, 8, 15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15,
    15, 15, 15, 15, 15, 15, 3, 15, 15, 8};

__constant__ uint8_t c_bc7_w[3][16] = {{0, 21, 43, 64}, {0, 9, 18, 27, 37, 46, 55, 64},
                                       {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64}};
// subsets, partition bits, rotation bits, index-selection bit, colour bits,
// alpha bits, p-bit per endpoint, p-bit per subset, index bits, second index bits
__constant__ uint8_t c_bc7_mode[8][10] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0}};

// n (<= 32) bits of the 128-bit block at bit `pos`, least significant first.
__device__ __forceinline__ uint32_t bc7_bits(uint64_t lo, uint64_t hi, uint32_t pos, uint32_t n) {
    if (n == 0) return 0u;
    uint64_t v;
    if (pos >= 64) v = hi >> (pos - 64);
    else if (pos == 0) v = lo;
    else v = (lo >> pos) | (hi << (64 - pos));
    return (uint32_t)(v & ((1ull << n) - 1ull));
}

__device__ __forceinline__ uint32_t bc7_expand(uint32_t v, uint32_t bits) {
    v <<= 8 - bits;
    return v | (v >> bits);
}

// The BC7 tables, copied into shared memory by each CTA: lanes of a warp
// decode blocks of different modes and partitions, and shared memory serves
// such scattered reads in one pass where the constant cache serialises them.
struct Bc7Tables {
    uint32_t p3[64];
    uint16_t p2[64];
    uint8_t a2[64], a3a[64], a3b[64];
    uint8_t w[3][16];
    uint8_t mode[8][10];
};

__device__ void bc7_load_tables(Bc7Tables& t) {
    for (uint32_t i = threadIdx.x; i < 64; i += blockDim.x) {
        t.p3[i] = c_bc7_p3[i];
        t.p2[i] = c_bc7_p2[i];
        t.a2[i] = c_bc7_a2[i];
        t.a3a[i] = c_bc7_a3a[i];
        t.a3b[i] = c_bc7_a3b[i];
    }
    for (uint32_t i = threadIdx.x; i < 48; i += blockDim.x) t.w[i / 16][i % 16] = c_bc7_w[i / 16][i % 16];
    for (uint32_t i = threadIdx.x; i < 80; i += blockDim.x) t.mode[i / 10][i % 10] = c_bc7_mode[i / 10][i % 10];
}

// Row r (4 texels) of one BC7 block, called by all 32 lanes together: the
// four lanes of a quad hold the same block (one row each) and share its end
// points, lane r unpacking end points r and r + 4 (RGBA8 after the p-bits and
// the bit replication) and the quad exchanging them by shuffles; then every
// texel selects its subset's pair.
__device__ void bc7_row(const Bc7Tables& T, const uint4& q, uint32_t r, uint32_t lane, uint32_t texel[4]) {
    const uint64_t lo = (uint64_t)q.x | ((uint64_t)q.y << 32), hi = (uint64_t)q.z | ((uint64_t)q.w << 32);
    const uint32_t first = q.x & 0xFFu;
    const bool reserved = first == 0;  // decodes to transparent black
    const uint32_t mode = reserved ? 0u : (uint32_t)(__ffs((int)first) - 1);
    const uint8_t* m = T.mode[mode];
    const uint32_t ns = m[0], cb = m[4], ab = m[5], ib = m[8], ib2 = m[9];
    uint32_t pos = mode + 1;
    const uint32_t part = bc7_bits(lo, hi, pos, m[1]);
    pos += m[1];
    const uint32_t rot = bc7_bits(lo, hi, pos, m[2]);
    pos += m[2];
    const uint32_t isel = bc7_bits(lo, hi, pos, m[3]);
    pos += m[3];
    // Stored fields in order: R of every end point (subset-major), then G,
    // B, then alpha, then the p-bits.  End point k = 2 s + e of channel c
    // starts at c_base[c] + k * bits.
    const uint32_t nep = 2 * ns;
    const uint32_t alpha_base = pos + 3 * nep * cb, pbit_base = alpha_base + nep * ab;
    const uint32_t cbits = cb + ((m[6] | m[7]) ? 1u : 0u);
    const uint32_t abits = ab ? ab + m[6] : 0u;
    uint32_t mine[2];  // this lane's end points r and r + 4, packed RGBA8
#pragma unroll
    for (uint32_t j = 0; j < 2; ++j) {
        const uint32_t k = r + 4 * j;
        mine[j] = 0u;
        if (k < nep) {
            // a p-bit per end point (modes 0, 3, 6, 7) or per subset (mode 1)
            const uint32_t pb = m[6] ? bc7_bits(lo, hi, pbit_base + k, 1) : (m[7] ? bc7_bits(lo, hi, pbit_base + k / 2, 1) : 0u);
            uint32_t v = 0u;
#pragma unroll
            for (uint32_t c = 0; c < 3; ++c) {
                uint32_t x = bc7_bits(lo, hi, pos + (c * nep + k) * cb, cb);
                if (m[6] | m[7]) x = (x << 1) | pb;
                v |= bc7_expand(x, cbits) << (8 * c);
            }
            uint32_t a = 255u;
            if (ab) {
                a = bc7_bits(lo, hi, alpha_base + k * ab, ab);
                if (m[6]) a = (a << 1) | pb;
                a = bc7_expand(a, abits);
            }
            mine[j] = v | (a << 24);
        }
    }
    uint32_t epk[6];  // packed RGBA8 of end point k, from lane k % 4 of the quad
#pragma unroll
    for (uint32_t k = 0; k < 6; ++k) epk[k] = __shfl_sync(0xffffffffu, mine[k >> 2], (lane & ~3u) | (k & 3u));
    const uint32_t a1 = ns == 2 ? T.a2[part] : (ns == 3 ? T.a3a[part] : 16u);
    const uint32_t a2 = ns == 3 ? T.a3b[part] : 16u;
    const uint32_t idx_start = pbit_base + (m[6] ? nep : (m[7] ? ns : 0u));
    const uint32_t idx2_start = idx_start + 16 * ib - ns;
    const uint32_t pmask = ns == 2 ? T.p2[part] : (ns == 3 ? T.p3[part] : 0u);
#pragma unroll
    for (uint32_t x = 0; x < 4; ++x) {
        const uint32_t i = 4 * r + x;
        const uint32_t s = ns == 1 ? 0u : (ns == 2 ? ((pmask >> i) & 1u) : ((pmask >> (2 * i)) & 3u));
        // anchors before texel i each store one bit less; an anchor itself too
        const uint32_t before = (i > 0 ? 1u : 0u) + (a1 < i ? 1u : 0u) + (a2 < i ? 1u : 0u);
        const bool anchor = i == 0 || i == a1 || i == a2;
        const uint32_t ix = bc7_bits(lo, hi, idx_start + i * ib - before, ib - (anchor ? 1u : 0u));
        uint32_t ci = ix, ai = ix, cw = ib, aw = ib;
        if (ib2) {
            const uint32_t ix2 = bc7_bits(lo, hi, idx2_start + i * ib2 - (i > 0 ? 1u : 0u), ib2 - (i == 0 ? 1u : 0u));
            if (isel) ci = ix2, cw = ib2;
            else ai = ix2, aw = ib2;
        }
        const uint32_t wc = T.w[cw - 2][ci], wa = T.w[aw - 2][ai];
        const uint32_t e0 = s == 0 ? epk[0] : (s == 1 ? epk[2] : epk[4]);
        const uint32_t e1 = s == 0 ? epk[1] : (s == 1 ? epk[3] : epk[5]);
        uint32_t px[4];
#pragma unroll
        for (uint32_t c = 0; c < 4; ++c) {
            const uint32_t w8 = c < 3 ? wc : wa;
            px[c] = ((64 - w8) * ((e0 >> (8 * c)) & 255u) + w8 * ((e1 >> (8 * c)) & 255u) + 32) >> 6;
        }
        if (rot) {  // swap alpha with R (1), G (2) or B (3)
            const uint32_t t = px[3];
            px[3] = px[rot - 1];
            px[rot - 1] = t;
        }
        texel[x] = reserved ? 0u : (px[0] | (px[1] << 8) | (px[2] << 16) | (px[3] << 24));
    }
}

// One block row of 4 texels from its block words.
__device__ __forceinline__ void decode_row(const uint4& q, uint32_t format, uint32_t r, uint32_t texel[4]) {
    if (format == VKGV_BC4 || format == VKGV_BC5) {
        uint32_t rr[4], gg[4] = {0, 0, 0, 0};
        channel_row(q.x, q.y, r, rr);
        if (format == VKGV_BC5) channel_row(q.z, q.w, r, gg);
#pragma unroll
        for (int x = 0; x < 4; ++x) texel[x] = rr[x] | (gg[x] << 8) | 0xFF000000u;
        return;
    }
    // colour block: words 0-1 (BC1) or 2-3 (BC2 / BC3, always four colours)
    const bool bc1 = format == VKGV_BC1 || format == VKGV_BC1_OPAQUE;
    const uint32_t clo = bc1 ? q.x : q.z, cidx = bc1 ? q.y : q.w;
    uint32_t pal[4];
    colour_palette(clo, bc1, format == VKGV_BC1_OPAQUE, pal);
    const uint32_t row = (cidx >> (8 * r)) & 255u;
#pragma unroll
    for (int x = 0; x < 4; ++x) texel[x] = pal[(row >> (2 * x)) & 3u];
    if (format == VKGV_BC2) {
        const uint32_t nib = ((r < 2 ? q.x : q.y) >> (16 * (r & 1u))) & 0xFFFFu;
#pragma unroll
        for (int x = 0; x < 4; ++x) texel[x] = (texel[x] & 0x00FFFFFFu) | ((((nib >> (4 * x)) & 15u) * 17u) << 24);
    } else if (format == VKGV_BC3) {
        uint32_t aa[4];
        channel_row(q.x, q.y, r, aa);
#pragma unroll
        for (int x = 0; x < 4; ++x) texel[x] = (texel[x] & 0x00FFFFFFu) | (aa[x] << 24);
    }
}

// Lane = 4 * (block in the warp's span of 8) + row in the block: the four
// lanes of a block share its (broadcast) load and each writes one row of 4
// texels (16 bytes when the row is inside the image).  Each thread handles
// kDecodeDepth block rows of y, with all their loads in flight first.
__global__ void __launch_bounds__(kDecodeWarps * 32) k_decode_bc(const uint8_t* __restrict__ blocks, uint32_t format,
                                                                 uint32_t w, uint32_t h, uint32_t* __restrict__ rgba) {
    pdl_begin();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t r = lane & 3u;
    const uint32_t bx = (blockIdx.x * kDecodeWarps + warp) * 8 + (lane >> 2);
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    if (bx >= bw) return;
    const bool wide = format != VKGV_BC1 && format != VKGV_BC4 && format != VKGV_BC1_OPAQUE;
    uint4 q[kDecodeDepth];
#pragma unroll
    for (int k = 0; k < kDecodeDepth; ++k) {
        const uint32_t by = blockIdx.y * kDecodeDepth + k;
        q[k] = make_uint4(0u, 0u, 0u, 0u);
        if (by < bh) {
            if (wide) {
                q[k] = __ldg(reinterpret_cast<const uint4*>(blocks) + ((size_t)by * bw + bx));
            } else {
                const uint2 v = __ldg(reinterpret_cast<const uint2*>(blocks) + ((size_t)by * bw + bx));
                q[k] = make_uint4(v.x, v.y, 0u, 0u);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kDecodeDepth; ++k) {
        const uint32_t y = (blockIdx.y * kDecodeDepth + k) * 4 + r;
        if (y >= h) break;
        uint32_t texel[4];
        decode_row(q[k], format, r, texel);
        uint32_t* dst = rgba + (size_t)y * w + (size_t)bx * 4;
        if (bx * 4 + 4 <= w && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            __stcs(reinterpret_cast<uint4*>(dst), make_uint4(texel[0], texel[1], texel[2], texel[3]));
        } else {
#pragma unroll
            for (int x = 0; x < 4; ++x)
                if (bx * 4 + x < w) __stcs(dst + x, texel[x]);
        }
    }
}

// BC7 with the lane layout of k_decode_bc (four lanes per block, one row
// each) and the tables in shared memory.  Every lane runs every step (the
// end points are shared by shuffles); lanes past the image edge decode a
// zero block and store nothing.
__global__ void __launch_bounds__(kDecodeWarps * 32) k_decode_bc7(const uint8_t* __restrict__ blocks, uint32_t w,
                                                                  uint32_t h, uint32_t* __restrict__ rgba) {
    __shared__ Bc7Tables T;
    bc7_load_tables(T);
    pdl_begin();
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t r = lane & 3u;
    const uint32_t bx = (blockIdx.x * kDecodeWarps + warp) * 8 + (lane >> 2);
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    uint4 q[kDecodeDepth];
#pragma unroll
    for (int k = 0; k < kDecodeDepth; ++k) {
        const uint32_t by = blockIdx.y * kDecodeDepth + k;
        q[k] = (bx < bw && by < bh) ? __ldg(reinterpret_cast<const uint4*>(blocks) + ((size_t)by * bw + bx))
                                    : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int k = 0; k < kDecodeDepth; ++k) {
        const uint32_t y = (blockIdx.y * kDecodeDepth + k) * 4 + r;
        uint32_t texel[4];
        bc7_row(T, q[k], r, lane, texel);
        if (bx >= bw || y >= h) continue;
        uint32_t* dst = rgba + (size_t)y * w + (size_t)bx * 4;
        if (bx * 4 + 4 <= w && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            __stcs(reinterpret_cast<uint4*>(dst), make_uint4(texel[0], texel[1], texel[2], texel[3]));
        } else {
#pragma unroll
            for (int x = 0; x < 4; ++x)
                if (bx * 4 + x < w) __stcs(dst + x, texel[x]);
        }
    }
}

// ------------------------------------------------------------------- BC6H
// BC6H (BPTC float; UF16 unsigned, SF16 signed) into float32 RGB (a linear
// VKGV_TEXTURE_RGB32F texture): the published format and the steps the
// oracle restates (oracle/texture.c), with the same partition, anchor and
// weight tables.  A 2-bit mode (values 0, 1) or a 5-bit one selects one of
// fourteen header layouts (the oracle's stream-order tokens regrouped by
// field, so that each field is assembled in its own register), transformed
// modes add signed
// deltas to the base endpoint, endpoints are unquantised to 16 bits, texels
// interpolated with the 3- or 4-bit BC7 weights and scaled to binary16
// (unsigned v * 31 >> 6; signed magnitude * 31 >> 5, sign only on a
// non-zero result).  Reserved modes decode to 0.  Four lanes per block, one
// row each, like k_decode_bc7; each lane parses the header itself.
// Header tokens grouped by field (endpoint w, x, y, z x channel R, G, B;
// 12 = partition), per mode: the bit position in the block (bits 0-6), the
// lowest field bit (7-10), bit count - 1 (11-14) and reversed (15: the first
// block bit is the highest field bit); the counts follow.
__constant__ uint16_t c_bc6_ftok[14][13][6] = {
    {{0x4805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x202D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2041, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0202, 0x1829, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0203, 0x183D, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2047, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0228, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0204, 0x0032, 0x00BC, 0x0146, 0x01CC, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x00
    {{0x3005, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x300F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3019, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x282D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2841, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0282, 0x0218, 0x1829, 0x0000, 0x0000, 0x0000}, {0x020E, 0x0296, 0x183D, 0x0000, 0x0000, 0x0000}, {0x2847, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0A03, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x080C, 0x0117, 0x01A0, 0x02A1, 0x0222, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x01
    {{0x4805, 0x0528, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0531, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x053B, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x182D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2041, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1829, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x183D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2047, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1833, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0032, 0x00BC, 0x0146, 0x01CC, 0x0000, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x02
    {{0x4805, 0x0527, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0532, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x053B, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x202D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1841, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1829, 0x024B, 0x0000, 0x0000, 0x0000, 0x0000}, {0x183D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1847, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0228, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x00BC, 0x0045, 0x0146, 0x01CC, 0x0000, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x06
    {{0x4805, 0x0527, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0531, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x053C, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x182D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1841, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1829, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0228, 0x183D, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1847, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1833, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0032, 0x08C5, 0x024B, 0x01CC, 0x0000, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x0A
    {{0x4005, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x400F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4019, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x202D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2041, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0218, 0x1829, 0x0000, 0x0000, 0x0000, 0x0000}, {0x020E, 0x183D, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2047, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0228, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0222, 0x0032, 0x00BC, 0x0146, 0x01CC, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x0E
    {{0x3805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x380F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x202D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2841, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0218, 0x1829, 0x0000, 0x0000, 0x0000, 0x0000}, {0x020E, 0x183D, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2847, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x020D, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0117, 0x09A1, 0x0032, 0x00BC, 0x0000, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x12
    {{0x3805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x380F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x282D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2041, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0297, 0x0218, 0x1829, 0x0000, 0x0000, 0x0000}, {0x020E, 0x183D, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2047, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x02A1, 0x0228, 0x1833, 0x0000, 0x0000, 0x0000}, {0x000D, 0x0222, 0x00BC, 0x0146, 0x01CC, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x16
    {{0x3805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x380F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x202D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2041, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0218, 0x1829, 0x0000, 0x0000, 0x0000, 0x0000}, {0x020E, 0x0297, 0x183D, 0x0000, 0x0000, 0x0000}, {0x2047, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0228, 0x1833, 0x0000, 0x0000, 0x0000, 0x0000}, {0x008D, 0x02A1, 0x0222, 0x0032, 0x0146, 0x01CC}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x1A
    {{0x2805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x280F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x282D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x2841, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0295, 0x0218, 0x1829, 0x0000, 0x0000, 0x0000}, {0x020E, 0x0296, 0x183D, 0x0000, 0x0000, 0x0000}, {0x2847, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x020B, 0x029F, 0x1833, 0x0000, 0x0000, 0x0000}, {0x080C, 0x0117, 0x01A0, 0x02A1, 0x0222, 0x0000}, {0x204D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x1E
    {{0x4805, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x482D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x03
    {{0x4805, 0x052C, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x0536, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x0540, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4023, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x402D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4037, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x07
    {{0x4805, 0x8D2B, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0x8D35, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0x8D3F, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x382D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x3837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x0B
    {{0x4805, 0xAD27, 0x0000, 0x0000, 0x0000, 0x0000}, {0x480F, 0xAD31, 0x0000, 0x0000, 0x0000, 0x0000}, {0x4819, 0xAD3B, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1823, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x182D, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x1837, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}, {0x0000, 0x0000, 0x0000, 0x0000, 0x0000, 0x0000}},  // mode 0x0F
};
__constant__ uint8_t c_bc6_fcount[14][13] = {
    {1, 1, 1, 1, 1, 1, 1, 2, 2, 1, 2, 5, 1},  // mode 0x00
    {1, 1, 1, 1, 1, 1, 1, 3, 3, 1, 2, 5, 1},  // mode 0x01
    {2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 4, 1},  // mode 0x02
    {2, 2, 2, 1, 1, 1, 1, 2, 1, 1, 2, 4, 1},  // mode 0x06
    {2, 2, 2, 1, 1, 1, 1, 1, 2, 1, 1, 4, 1},  // mode 0x0A
    {1, 1, 1, 1, 1, 1, 1, 2, 2, 1, 2, 5, 1},  // mode 0x0E
    {1, 1, 1, 1, 1, 1, 1, 2, 2, 1, 2, 4, 1},  // mode 0x12
    {1, 1, 1, 1, 1, 1, 1, 3, 2, 1, 3, 5, 1},  // mode 0x16
    {1, 1, 1, 1, 1, 1, 1, 2, 3, 1, 2, 6, 1},  // mode 0x1A
    {1, 1, 1, 1, 1, 1, 1, 3, 3, 1, 3, 5, 1},  // mode 0x1E
    {1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0},  // mode 0x03
    {2, 2, 2, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0},  // mode 0x07
    {2, 2, 2, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0},  // mode 0x0B
    {2, 2, 2, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0},  // mode 0x0F
};
// mode value, transformed, endpoint bits, delta bits R, G, B, regions, tokens
// (the oracle's stream-order count)
__constant__ uint8_t c_bc6_mode[14][8] = {
    {0x00, 1, 10, 5, 5, 5, 2, 20}, {0x01, 1, 7, 6, 6, 6, 2, 22},   {0x02, 1, 11, 5, 4, 4, 2, 19},
    {0x06, 1, 11, 4, 5, 4, 2, 21}, {0x0A, 1, 11, 4, 4, 5, 2, 20},  {0x0E, 1, 9, 5, 5, 5, 2, 20},
    {0x12, 1, 8, 6, 5, 5, 2, 19},  {0x16, 1, 8, 5, 6, 5, 2, 22},   {0x1A, 1, 8, 5, 5, 6, 2, 22},
    {0x1E, 0, 6, 6, 6, 6, 2, 23},  {0x03, 0, 10, 10, 10, 10, 1, 6}, {0x07, 1, 11, 9, 9, 9, 1, 9},
    {0x0B, 1, 12, 8, 8, 8, 1, 9},  {0x0F, 1, 16, 4, 4, 4, 1, 9}};

struct Bc6Tables {
    uint16_t ftok[14][13][6];
    uint8_t fcount[14][13];
    uint8_t mode[14][8];
    int8_t row[32];  // 5-bit mode field -> mode row, -1 for a reserved mode
    uint16_t p2[32];
    uint8_t a2[32];
    uint8_t w3[8], w4[16];
};

__device__ void bc6_load_tables(Bc6Tables& t) {
    for (uint32_t i = threadIdx.x; i < 14 * 13 * 6; i += blockDim.x)
        t.ftok[i / 78][(i / 6) % 13][i % 6] = c_bc6_ftok[i / 78][(i / 6) % 13][i % 6];
    for (uint32_t i = threadIdx.x; i < 14 * 13; i += blockDim.x) t.fcount[i / 13][i % 13] = c_bc6_fcount[i / 13][i % 13];
    for (uint32_t i = threadIdx.x; i < 14 * 8; i += blockDim.x) t.mode[i / 8][i % 8] = c_bc6_mode[i / 8][i % 8];
    for (uint32_t i = threadIdx.x; i < 32; i += blockDim.x) {
        // a field whose two low bits are 0 or 1 is a 2-bit mode
        const uint32_t m = (i & 3u) < 2u ? (i & 3u) : i;
        int8_t r = -1;
        for (int k = 0; k < 14; ++k)
            if (c_bc6_mode[k][0] == m) r = (int8_t)k;
        t.row[i] = r;
        t.p2[i] = c_bc7_p2[i];
        t.a2[i] = c_bc7_a2[i];
    }
    for (uint32_t i = threadIdx.x; i < 8; i += blockDim.x) t.w3[i] = c_bc7_w[1][i];
    for (uint32_t i = threadIdx.x; i < 16; i += blockDim.x) t.w4[i] = c_bc7_w[2][i];
}

__device__ __forceinline__ int32_t bc6_sext(uint32_t v, uint32_t n) {
    const uint32_t s = 32u - n;
    return (int32_t)(v << s) >> s;
}

__device__ __forceinline__ int32_t bc6_unquantize(int32_t c, uint32_t bits, bool sgn) {
    if (!sgn) {
        if (bits >= 15u) return c;
        if (c == 0) return 0;
        if (c == (int32_t)((1u << bits) - 1u)) return 0xFFFF;
        return (int32_t)((((uint32_t)c << 16) + 0x8000u) >> bits);
    }
    if (bits >= 16u) return c;
    const bool neg = c < 0;
    const int32_t m = neg ? -c : c;
    int32_t u;
    if (m == 0) u = 0;
    else if (m >= (int32_t)((1u << (bits - 1u)) - 1u)) u = 0x7FFF;
    else u = (int32_t)((((uint32_t)m << 15) + 0x4000u) >> (bits - 1u));
    return neg ? -u : u;
}

__device__ __forceinline__ uint16_t bc6_finish(int32_t v, bool sgn) {
    if (!sgn) return (uint16_t)((v * 31) >> 6);
    if (v < 0) {
        const int32_t m = ((-v) * 31) >> 5;
        return (uint16_t)(m ? (m | 0x8000) : 0);
    }
    return (uint16_t)((v * 31) >> 5);
}

// Row r (4 texels, R, G, B as float32) of one BC6H block.
__device__ __forceinline__ void bc6_row(const Bc6Tables& T, const uint4& q, uint32_t r, bool sgn, float out[12]) {
    const uint64_t lo = (uint64_t)q.x | ((uint64_t)q.y << 32), hi = (uint64_t)q.z | ((uint64_t)q.w << 32);
    const int mi = T.row[q.x & 31u];
    if (mi < 0) {
#pragma unroll
        for (int k = 0; k < 12; ++k) out[k] = 0.0f;
        return;
    }
    const uint8_t* M = T.mode[mi];
    uint32_t f[13];
#pragma unroll
    for (int k = 0; k < 13; ++k) {
        uint32_t acc = 0u;
        for (uint32_t t = 0; t < T.fcount[mi][k]; ++t) {
            const uint32_t tok = T.ftok[mi][k][t], n = ((tok >> 11) & 15u) + 1u;
            uint32_t v = bc7_bits(lo, hi, tok & 127u, n);
            if (tok >> 15) v = __brev(v) >> (32u - n);
            acc |= v << ((tok >> 7) & 15u);
        }
        f[k] = acc;
    }
    // the header ends after the partition field (two regions) or the
    // last end point (one region)
    const uint32_t pos = M[6] == 2u ? 82u : 65u;
    const bool tr = M[1] != 0;
    const uint32_t bits = M[2], ns = M[6];
    int32_t ep[4][3];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint32_t raw = f[e * 3 + c];
            int32_t v;
            if (e == 0 || !tr) {
                v = sgn ? bc6_sext(raw, bits) : (int32_t)raw;
            } else {
                const uint32_t sum = (f[c] + (uint32_t)bc6_sext(raw, M[3 + c])) & ((1u << bits) - 1u);
                v = sgn ? bc6_sext(sum, bits) : (int32_t)sum;
            }
            ep[e][c] = bc6_unquantize(v, bits, sgn);
        }
    const uint32_t part = f[12] & 31u, anchor = ns == 2u ? T.a2[part] : 16u, ib = ns == 2u ? 3u : 4u;
    // index bits of texels 4r .. 4r + 3: the header, then ib bits a texel,
    // one less for texel 0 and the second region's anchor
    uint32_t ipos = pos + 4u * r * ib - (r > 0 ? 1u : 0u) - ((anchor < 4u * r) ? 1u : 0u);
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const uint32_t i = 4u * r + (uint32_t)x;
        const uint32_t n = ib - ((i == 0u || i == anchor) ? 1u : 0u);
        const uint32_t idx = bc7_bits(lo, hi, ipos, n);
        ipos += n;
        const uint32_t s = ns == 2u ? ((T.p2[part] >> i) & 1u) : 0u;
        const int32_t w = ns == 2u ? T.w3[idx] : T.w4[idx];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int32_t e0 = s ? ep[2][c] : ep[0][c], e1 = s ? ep[3][c] : ep[1][c];
            const int32_t v = ((64 - w) * e0 + w * e1 + 32) >> 6;  // arithmetic: floor division
            out[3 * x + c] = __half2float(__ushort_as_half(bc6_finish(v, sgn)));
        }
    }
}

__global__ void __launch_bounds__(kDecodeWarps * 32) k_decode_bc6h(const uint8_t* __restrict__ blocks, uint32_t w,
                                                                   uint32_t h, uint32_t is_signed,
                                                                   float* __restrict__ rgb) {
    __shared__ Bc6Tables T;
    bc6_load_tables(T);
    pdl_begin();
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t r = lane & 3u;
    const uint32_t bx = (blockIdx.x * kDecodeWarps + warp) * 8 + (lane >> 2);
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    const bool sgn = is_signed != 0;
    // the header parse dominates, so each block row is loaded when needed
#pragma unroll 1
    for (int k = 0; k < kDecodeDepth; ++k) {
        const uint32_t by = blockIdx.y * kDecodeDepth + k, y = by * 4 + r;
        if (bx >= bw || by >= bh || y >= h) continue;
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(blocks) + ((size_t)by * bw + bx));
        float t[12];
        bc6_row(T, q, r, sgn, t);
        float* dst = rgb + ((size_t)y * w + (size_t)bx * 4) * 3;
        if (bx * 4 + 4 <= w && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            float4* d4 = reinterpret_cast<float4*>(dst);
            __stcs(d4, make_float4(t[0], t[1], t[2], t[3]));
            __stcs(d4 + 1, make_float4(t[4], t[5], t[6], t[7]));
            __stcs(d4 + 2, make_float4(t[8], t[9], t[10], t[11]));
        } else {
            for (uint32_t x = 0; x < 4 && bx * 4 + x < w; ++x)
#pragma unroll
                for (int c = 0; c < 3; ++c) __stcs(dst + 3 * x + c, t[3 * x + c]);
        }
    }
}

// ------------------------------------------------------------------- JPEG
// The device half of a JPEG decode (the host half, jpeg.cpp, writes the
// dequantized coefficient planes).  Pinned fixed-point arithmetic, shared
// with the oracle:
//   IDCT: K[x][u] = round(8192 * c(u) / 2 * cos((2x + 1) u pi / 16)),
//     c(0) = 1 / sqrt(2), c(u > 0) = 1; rows t[v][x] = (sum_u K[x][u] F[v][u]
//     + 512) >> 10 (int32, 3 fractional bits kept), then columns
//     s[y][x] = (sum_v K[y][v] t[v][x] + 2^15) >> 16 (int64), + 128, clamped
//     to 0..255; right shifts are arithmetic.
//   upsampling: component c at pixel (x, y) is its sample
//     (x / (hmax / h_c), y / (vmax / v_c)) (replication).
//   YCbCr -> RGB (JFIF): with cb = Cb - 128, cr = Cr - 128,
//     R = Y + ((91881 cr + 32768) >> 16),
//     G = Y + ((-22554 cb - 46802 cr + 32768) >> 16),
//     B = Y + ((116130 cb + 32768) >> 16), each clamped to 0..255.

__constant__ int32_t c_idct[8][8] = {
    {2896, 4017, 3784, 3406, 2896, 2276, 1567, 799},     {2896, 3406, 1567, -799, -2896, -4017, -3784, -2276},
    {2896, 2276, -1567, -4017, -2896, 799, 3784, 3406},  {2896, 799, -3784, -2276, 2896, 3406, -1567, -4017},
    {2896, -799, -3784, 2276, 2896, -3406, -1567, 4017}, {2896, -2276, -1567, 4017, -2896, -799, 3784, -3406},
    {2896, -3406, 1567, 799, -2896, 4017, -3784, 2276},  {2896, -4017, 3784, -3406, 2896, -2276, 1567, -799},
};

constexpr int kIdctBlocks = 32;  // 8x8 blocks per CTA, one thread per block row

// Coefficient blocks (raster order over a blocks_w-wide grid) -> 8-bit
// samples of a (blocks_w * 8)-wide plane.
__global__ void __launch_bounds__(kIdctBlocks * 8) k_jpeg_idct(const int16_t* __restrict__ coef, uint32_t blocks,
                                                               uint32_t blocks_w, uint8_t* __restrict__ plane) {
    pdl_begin();
    __shared__ int32_t t[kIdctBlocks][8][9];
    const uint32_t local = threadIdx.x >> 3, r = threadIdx.x & 7u;
    const uint32_t b = blockIdx.x * kIdctBlocks + local;
    const bool live = b < blocks;
    if (live) {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(coef + (size_t)b * 64 + r * 8));
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
        int32_t f[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            f[2 * i] = int32_t(int16_t(w[i] & 0xFFFFu));
            f[2 * i + 1] = int32_t(int16_t(w[i] >> 16));
        }
#pragma unroll
        for (int x = 0; x < 8; ++x) {
            int32_t acc = 0;
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += c_idct[x][u] * f[u];
            t[local][r][x] = (acc + 512) >> 10;
        }
    }
    __syncthreads();
    if (!live) return;
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int x = 0; x < 8; ++x) {
        int64_t acc = 0;
#pragma unroll
        for (int v = 0; v < 8; ++v) acc += int64_t(c_idct[r][v]) * t[local][v][x];
        const int32_t s = min(255, max(0, int32_t((acc + 32768) >> 16) + 128));
        if (x < 4) lo |= uint32_t(s) << (8 * x);
        else hi |= uint32_t(s) << (8 * (x - 4));
    }
    const uint32_t bx = b % blocks_w, by = b / blocks_w;
    *reinterpret_cast<uint2*>(plane + ((size_t)by * 8 + r) * ((size_t)blocks_w * 8) + (size_t)bx * 8) = make_uint2(lo, hi);
}

__global__ void __launch_bounds__(256) k_jpeg_color(JpegPlanes P, uint32_t* __restrict__ rgba) {
    pdl_begin();
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31u), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= P.width || y >= P.height) return;
    int32_t c[3] = {0, 0, 0};
#pragma unroll
    for (uint32_t k = 0; k < 3; ++k)  // constant indices keep the parameters out of local memory
        if (k < P.components) c[k] = P.plane[k][(size_t)(y / P.ry[k]) * P.pitch[k] + x / P.rx[k]];
    uint32_t r, g, b;
    if (P.components == 1) {
        r = g = b = uint32_t(c[0]);
    } else if (P.rgb) {
        r = uint32_t(c[0]);
        g = uint32_t(c[1]);
        b = uint32_t(c[2]);
    } else {
        const int32_t cb = c[1] - 128, cr = c[2] - 128;
        r = uint32_t(min(255, max(0, c[0] + ((91881 * cr + 32768) >> 16))));
        g = uint32_t(min(255, max(0, c[0] + ((-22554 * cb - 46802 * cr + 32768) >> 16))));
        b = uint32_t(min(255, max(0, c[0] + ((116130 * cb + 32768) >> 16))));
    }
    rgba[(size_t)y * P.width + x] = r | (g << 8) | (b << 16) | 0xFF000000u;
}

}  // namespace

void launch_jpeg_idct(const int16_t* coef, uint32_t blocks_w, uint32_t blocks_h, uint8_t* plane, cudaStream_t stream) {
    const uint32_t blocks = blocks_w * blocks_h;
    launch_pdl(k_jpeg_idct, dim3((blocks + kIdctBlocks - 1) / kIdctBlocks), dim3(kIdctBlocks * 8), 0, stream, coef,
               blocks, blocks_w, plane);
}

void launch_jpeg_color(const JpegPlanes& P, uint32_t* rgba, cudaStream_t stream) {
    launch_pdl(k_jpeg_color, dim3((P.width + 31) / 32, (P.height + 7) / 8), dim3(256), 0, stream, P, rgba);
}

void launch_decode_bc6h(const uint8_t* blocks, bool is_signed, uint32_t w, uint32_t h, float* rgb,
                        cudaStream_t stream) {
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    const uint32_t per_cta = 8 * kDecodeWarps;
    const dim3 grid((bw + per_cta - 1) / per_cta, (bh + kDecodeDepth - 1) / kDecodeDepth);
    launch_pdl(k_decode_bc6h, grid, dim3(kDecodeWarps * 32), 0, stream, blocks, w, h, is_signed ? 1u : 0u, rgb);
}

void launch_decode_bc(const uint8_t* blocks, uint32_t format, uint32_t w, uint32_t h, uint32_t* rgba,
                      cudaStream_t stream) {
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    const uint32_t per_cta = 8 * kDecodeWarps;
    const dim3 grid((bw + per_cta - 1) / per_cta, (bh + kDecodeDepth - 1) / kDecodeDepth);
    if (format == VKGV_BC7)
        launch_pdl(k_decode_bc7, grid, dim3(kDecodeWarps * 32), 0, stream, blocks, w, h, rgba);
    else
        launch_pdl(k_decode_bc, grid, dim3(kDecodeWarps * 32), 0, stream, blocks, format, w, h, rgba);
}

}  // namespace vkgv
