// Block-compressed texture decode on the device: BC1-BC5 (the DXT1-5 /
// RGTC formats a DDS base-colour texture holds, MSFT_texture_dds) into RGBA8
// for the textured resolve.  The reference loads no images
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

void launch_decode_bc(const uint8_t* blocks, uint32_t format, uint32_t w, uint32_t h, uint32_t* rgba,
                      cudaStream_t stream) {
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    const uint32_t per_cta = 8 * kDecodeWarps;
    launch_pdl(k_decode_bc, dim3((bw + per_cta - 1) / per_cta, (bh + kDecodeDepth - 1) / kDecodeDepth),
               dim3(kDecodeWarps * 32), 0, stream, blocks, format, w, h, rgba);
}

}  // namespace vkgv
