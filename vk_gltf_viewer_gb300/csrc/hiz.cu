// HiZ min-pyramid: the reduce chain of application.cpp:951-1003 that runs
// shaders/hiz_reduce.comp.glsl once per level, here in one launch per frame.
//
// Level i (1..L) writes mip i-1 at size (W>>i, H>>i) from mip i-2 (the depth
// image for i = 1): texel p = MIN over the bilinear footprint of the source
// at ((p + 0.5) / size) with clamp-to-edge (the MIN-reduction sampler of
// application.cpp:437-458).  Where (W>>i, H>>i) has a zero dimension the
// reference dispatches no work and the mip stays undefined; it is defined
// here as 0.0 (far plane under reverse-Z, so it never occludes).  The
// reference's bounds test `pos > size` (hiz_reduce.comp.glsl:24) also lets
// pos == size through, whose image store is out of bounds; only pos < size is
// written here.
//
// Single pass: each CTA owns a 4x4 tile of level 4 and the 8x8, 16x16 and
// 32x32 tiles of levels 3, 2, 1 above it (510 CTAs of 256 threads at
// 1920x1080, several resident per SM).  For odd sizes the footprints do
// not nest, so each CTA computes the hull of its owned tile and the
// footprint of the level above it (a halo of a few texels, recomputed rather
// than exchanged), keeping levels 1-3 in shared memory and reading the depth
// image once.  The last CTA of a view to finish computes the remaining top
// levels: the footprints of all their columns and rows in one table, the
// first of them from the top tiled mip in L2, the rest from shared memory
// with one barrier per level.
#include <atomic>

#include "kernels.cuh"

namespace vkgv {

namespace {

// Per-axis shared-memory capacity per tile level: the owned tile (32, 16,
// 8, 4 texels) plus the footprint of the level above it, which for odd
// sizes reaches one texel further per level.
constexpr int kCap1 = 48, kCap2 = 26, kCap3 = 14, kCap4 = 8;
constexpr int kThreads = 256;
// Dynamic shared memory: the tile levels, later reused by the tail's levels
// when they fit kTailMax floats; the launch sizes it to the larger of the
// two uses.
constexpr int kOff2 = kCap1 * kCap1, kOff3 = kOff2 + kCap2 * kCap2, kOff4 = kOff3 + kCap3 * kCap3;
constexpr int kTileFloats = kOff4 + kCap4 * kCap4;
constexpr int kTailMax = 40960;
constexpr int kTailAxis = 1024;  // footprint-table entries per axis over all tail levels
#ifndef VKGV_HIZ_TAIL_BATCH
#define VKGV_HIZ_TAIL_BATCH 2
#endif
constexpr int kTailBatch = VKGV_HIZ_TAIL_BATCH;  // first tail level: texels per thread with loads in flight

struct Range {
    int lo, hi;  // inclusive; empty when lo > hi
};

__device__ __forceinline__ Range hull(Range a, Range b) {
    if (a.lo > a.hi) return b;
    if (b.lo > b.hi) return a;
    return Range{min(a.lo, b.lo), max(a.hi, b.hi)};
}

// Texels of level j (size s_lo) read by texels [r.lo, r.hi] of level j+1
// (size s_hi); the footprint is monotone in the texel index.
__device__ __forceinline__ Range footprint_range(Range r, uint32_t s_hi, uint32_t s_lo) {
    if (r.lo > r.hi) return r;
    if (s_lo == 2 * s_hi) return Range{2 * r.lo, 2 * r.hi + 1};  // exact halving (see axis_footprint)
    int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
    footprint_axis(fdiv(fadd((float)r.lo, 0.5f), (float)s_hi), s_lo, a0, a1);
    const int nb = footprint_axis(fdiv(fadd((float)r.hi, 0.5f), (float)s_hi), s_lo, b0, b1);
    return Range{a0, nb == 2 ? b1 : b0};
}

__device__ __forceinline__ Range owned(uint32_t tile, uint32_t t, uint32_t size) {
    const int lo = (int)(tile * t);
    const int hi = (int)min((tile + 1) * t, size) - 1;
    return Range{lo, hi};
}

__device__ __forceinline__ float depth_at(const unsigned long long* d, uint32_t w, int x, int y) {
    return u2f((uint32_t)(__ldg(d + (size_t)y * w + x) >> 32));
}

// Footprint along one axis of texel x of a level of size d in its source of
// size s.  When s == 2d the sample point (x + 0.5) / d * s - 0.5 lies within
// about (2x + 1) * 2^-22 of 2x + 0.5 (sizes <= 8192), so both weights are
// non-zero and the footprint is exactly {2x, 2x + 1}: no division needed.
__device__ __forceinline__ int axis_footprint(int x, uint32_t d, uint32_t s, int& i0, int& i1) {
    if (s == 2 * d) {
        i0 = 2 * x;
        i1 = 2 * x + 1;
        return 2;
    }
    return footprint_axis(fdiv(fadd((float)x, 0.5f), (float)d), s, i0, i1);
}

// One texel of level j from a source sampled through `fetch(x, y)`.
template <class F>
__device__ __forceinline__ float reduce_texel(int x, int y, uint32_t dw, uint32_t dh, uint32_t sw, uint32_t sh,
                                              F fetch) {
    int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
    const int nx = axis_footprint(x, dw, sw, x0, x1);
    const int ny = axis_footprint(y, dh, sh, y0, y1);
    float r = fetch(x0, y0);
    if (nx == 2) r = gmin(r, fetch(x1, y0));
    if (ny == 2) {
        r = gmin(r, fetch(x0, y1));
        if (nx == 2) r = gmin(r, fetch(x1, y1));
    }
    return r;
}

__global__ void __launch_bounds__(kThreads, 5) k_hiz(const DeviceView* __restrict__ views, uint32_t* status,
                                                  uint32_t tail) {
    pdl_begin();
    const DeviceView& V = views[blockIdx.z];
    if (!V.pyr || V.pyr_levels == 0) return;
    const uint32_t w = V.w, h = V.h, L = V.pyr_levels;
    const uint32_t w0 = w >> 1, h0 = h >> 1;
    const int Kp = hiz_tile_levels(w, h, L);
    uint32_t ntx = 1, nty = 1;
    hiz_tiles(w, h, L, &ntx, &nty);
    const uint32_t bx = blockIdx.x, by = blockIdx.y;
    if (bx >= ntx || by >= nty) return;

    extern __shared__ float smem[];
    __shared__ Range rx[5], ry[5];
    __shared__ int s_bad, s_last;
    float* lvl[5] = {nullptr, smem, smem + kOff2, smem + kOff3, smem + kOff4};
    const int cap[5] = {0, kCap1, kCap2, kCap3, kCap4};

    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    if (threadIdx.x == 0 || threadIdx.x == 32) {
        // Ranges each level must compute along one axis (x by thread 0, y
        // by thread 32): the owned tile, plus the footprint of the level
        // above (top-down).
        const bool ax = threadIdx.x == 0;
        const uint32_t full = ax ? w : h, b = ax ? bx : by;
        Range* rr = ax ? rx : ry;
        for (int j = Kp; j >= 1; --j) {
            const uint32_t t = (uint32_t)hiz_tile_edge(j, Kp);
            Range o = owned(b, t, full >> j);
            if (j < Kp) o = hull(o, footprint_range(rr[j + 1], full >> (j + 1), full >> j));
            rr[j] = o;
            if (o.hi - o.lo + 1 > cap[j]) s_bad = 1;
        }
    }
    __syncthreads();
    if (s_bad) {
        if (threadIdx.x == 0) report(status, kStatusBadIndex, 0x48495a00u | (uint32_t)Kp);
    } else {
        for (int j = 1; j <= Kp; ++j) {
            const Range X = rx[j], Y = ry[j];
            const int rw = X.hi - X.lo + 1, rh = Y.hi - Y.lo + 1;
            if (rw <= 0 || rh <= 0) {
                __syncthreads();
                continue;
            }
            const uint32_t dw = w >> j, dh = h >> j;
            const uint32_t t = (uint32_t)hiz_tile_edge(j, Kp);
            const Range OX = owned(bx, t, dw), OY = owned(by, t, dh);
            float* dst = V.pyr + mip_offset(w0, h0, (uint32_t)(j - 1));
            float* here = lvl[j];
            const float* below = lvl[j - 1];
            const Range BX = j > 1 ? rx[j - 1] : Range{0, 0};
            const Range BY = j > 1 ? ry[j - 1] : Range{0, 0};
            const int bw = BX.hi - BX.lo + 1;
            if (j == 1 && w == 2 * dw && h == 2 * dh) {
                // Level 1 over the depth image, 2x2 blocks with one 16-byte
                // load per row (depth_id is 16-byte aligned and w is even).
                // Batches of four texels per thread: all eight loads are in
                // flight before the first minimum.
                for (int i0 = threadIdx.x; i0 < rw * rh; i0 += 4 * kThreads) {
                    uint32_t d[4][4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int i = i0 + k * kThreads;
                        if (i < rw * rh) {
                            const int x = X.lo + i % rw, y = Y.lo + i / rw;
                            const ulonglong2* q =
                                reinterpret_cast<const ulonglong2*>(V.depth_id + (size_t)(2 * y) * w + 2 * x);
                            const ulonglong2 a = __ldg(q), b = __ldg(q + (w >> 1));
                            d[k][0] = (uint32_t)(a.x >> 32), d[k][1] = (uint32_t)(a.y >> 32);
                            d[k][2] = (uint32_t)(b.x >> 32), d[k][3] = (uint32_t)(b.y >> 32);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int i = i0 + k * kThreads;
                        if (i < rw * rh) {
                            const int x = X.lo + i % rw, y = Y.lo + i / rw;
                            const float r = gmin(gmin(gmin(u2f(d[k][0]), u2f(d[k][1])), u2f(d[k][2])), u2f(d[k][3]));
                            here[i] = r;
                            if (x >= OX.lo && x <= OX.hi && y >= OY.lo && y <= OY.hi) dst[(size_t)y * dw + x] = r;
                        }
                    }
                }
                __syncthreads();
                continue;
            }
#pragma unroll 4
            for (int i = threadIdx.x; i < rw * rh; i += blockDim.x) {
                const int x = X.lo + i % rw, y = Y.lo + i / rw;
                float r;
                if (j == 1) {
                    r = reduce_texel(x, y, dw, dh, w, h, [&](int sx, int sy) { return depth_at(V.depth_id, w, sx, sy); });
                } else {
                    r = reduce_texel(x, y, dw, dh, w >> (j - 1), h >> (j - 1),
                                     [&](int sx, int sy) { return below[(sy - BY.lo) * bw + (sx - BX.lo)]; });
                }
                here[i] = r;
                if (x >= OX.lo && x <= OX.hi && y >= OY.lo && y <= OY.hi) dst[(size_t)y * dw + x] = r;
            }
            __syncthreads();
        }
    }
    // The last CTA of this view finishes levels Kp+1..L.
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&V.counters[3], 1u) == ntx * nty - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t top_w = Kp > 0 ? (w >> Kp) : 0, top_h = Kp > 0 ? (h >> Kp) : 0;
    const uint32_t next_px = Kp > 0 ? (w >> (Kp + 1)) * (h >> (Kp + 1)) : 0;
    // Levels Kp+1..Lv have both dimensions non-zero; the ones above are 0.
    uint32_t Lv = (uint32_t)Kp, sum_w = 0, sum_h = 0, sum_px = 0;
    while (Lv < L && (w >> (Lv + 1)) != 0 && (h >> (Lv + 1)) != 0) {
        ++Lv;
        sum_w += w >> Lv;
        sum_h += h >> Lv;
        sum_px += (w >> Lv) * (h >> Lv);
    }
    // Shared-memory tail: the footprints of every column and row of every
    // tail level are tabulated in one pass; level Kp+1 reads the top tiled
    // mip straight from L2 (a thread's loads in flight together), each level
    // above it reads the previous one from shared memory with one barrier
    // per level, and all of them are written out at the end in one pass.
    // (Written out level by level, the tail of a 1080p view took 8 us, more
    // than the 7.3 us of all its tiles.)
    __shared__ uint32_t s_fx[kTailAxis], s_fy[kTailAxis];
    const bool fast = Kp > 0 && Lv > (uint32_t)Kp && sum_px <= tail && sum_w <= (uint32_t)kTailAxis &&
                      sum_h <= (uint32_t)kTailAxis;
    uint32_t first_zero = (uint32_t)Kp + 1;
    if (fast) {
        // entry: x0 | x1 << 14 | n << 28 (x1 = x0 when n = 1)
        for (uint32_t i = threadIdx.x; i < sum_w + sum_h; i += blockDim.x) {
            const bool isx = i < sum_w;
            const uint32_t full = isx ? w : h;
            uint32_t k = isx ? i : i - sum_w, j = (uint32_t)Kp + 1;
            while (k >= (full >> j)) {
                k -= full >> j;
                ++j;
            }
            int a = 0, b = 0;
            const int n = axis_footprint((int)k, full >> j, full >> (j - 1), a, b);
            if (n == 1) b = a;
            const uint32_t packed = (uint32_t)a | ((uint32_t)b << 14) | ((uint32_t)n << 28);
            if (isx) s_fx[i] = packed;
            else s_fy[i - sum_w] = packed;
        }
        __syncthreads();
        // levels Kp+1..Lv stay in shared memory, contiguous as in the pyramid
        float* lv = smem;
        const uint64_t base = mip_offset(w0, h0, (uint32_t)Kp);  // level Kp+1
        {
            const float* src = V.pyr + (base - (uint64_t)top_w * top_h);  // the top tiled mip
            const uint32_t dw = w >> (Kp + 1), sw = top_w, n = next_px;
            for (uint32_t i0 = threadIdx.x; i0 < n; i0 += kTailBatch * kThreads) {
                float t[kTailBatch][4];
                uint32_t two[kTailBatch];
#pragma unroll
                for (int k = 0; k < kTailBatch; ++k) {
                    const uint32_t i = i0 + (uint32_t)k * kThreads;
                    if (i < n) {
                        const uint32_t y = i / dw, x = i - y * dw;
                        const uint32_t fx = s_fx[x], fy = s_fy[y];
                        const uint32_t x0 = fx & 0x3fffu, x1 = (fx >> 14) & 0x3fffu;
                        const uint32_t r0 = (fy & 0x3fffu) * sw, r1 = ((fy >> 14) & 0x3fffu) * sw;
                        two[k] = (fx >> 28) | ((fy >> 28) << 2);
                        t[k][0] = __ldcg(src + r0 + x0);
                        t[k][1] = __ldcg(src + r0 + x1);
                        t[k][2] = __ldcg(src + r1 + x0);
                        t[k][3] = __ldcg(src + r1 + x1);
                    }
                }
#pragma unroll
                for (int k = 0; k < kTailBatch; ++k) {
                    const uint32_t i = i0 + (uint32_t)k * kThreads;
                    if (i < n) {
                        const bool nx2 = (two[k] & 3u) == 2u, ny2 = (two[k] >> 2) == 2u;
                        float r = t[k][0];
                        if (nx2) r = gmin(r, t[k][1]);
                        if (ny2) {
                            r = gmin(r, t[k][2]);
                            if (nx2) r = gmin(r, t[k][3]);
                        }
                        lv[i] = r;
                    }
                }
            }
        }
        __syncthreads();
        uint32_t ox = w >> (Kp + 1), oy = h >> (Kp + 1), so = 0, sz = next_px;
        for (uint32_t j = (uint32_t)Kp + 2; j <= Lv; ++j) {
            const uint32_t dw = w >> j, dh = h >> j, sw = w >> (j - 1);
            const float* cur = lv + so;
            float* nxt = lv + so + sz;
            for (uint32_t i = threadIdx.x; i < dw * dh; i += kThreads) {
                const uint32_t y = i / dw, x = i - y * dw;
                const uint32_t fx = s_fx[ox + x], fy = s_fy[oy + y];
                const uint32_t x0 = fx & 0x3fffu, x1 = (fx >> 14) & 0x3fffu;
                const uint32_t r0 = (fy & 0x3fffu) * sw, r1 = ((fy >> 14) & 0x3fffu) * sw;
                const bool nx2 = (fx >> 28) == 2u, ny2 = (fy >> 28) == 2u;
                float r = cur[r0 + x0];
                if (nx2) r = gmin(r, cur[r0 + x1]);
                if (ny2) {
                    r = gmin(r, cur[r1 + x0]);
                    if (nx2) r = gmin(r, cur[r1 + x1]);
                }
                nxt[i] = r;
            }
            so += sz;
            sz = dw * dh;
            ox += dw;
            oy += dh;
            __syncthreads();
        }
        // every tail level out in one coalesced pass
        float* dst = V.pyr + base;
        for (uint32_t i = threadIdx.x; i < so + sz; i += kThreads) dst[i] = lv[i];
        first_zero = Lv + 1;
    }
    // Otherwise each texel reads its footprint from global memory.
    for (uint32_t j = first_zero; j <= L; ++j) {
        const uint32_t dw = w >> j, dh = h >> j;
        const uint32_t mw = mip_dim(w0, j - 1), mh = mip_dim(h0, j - 1);
        float* dst = V.pyr + mip_offset(w0, h0, j - 1);
        if (dw == 0 || dh == 0) {
            for (uint32_t i = threadIdx.x; i < mw * mh; i += blockDim.x) dst[i] = 0.0f;
        } else {
            const uint32_t sw = j == 1 ? w : mip_dim(w0, j - 2), sh = j == 1 ? h : mip_dim(h0, j - 2);
            const float* src = j == 1 ? nullptr : V.pyr + mip_offset(w0, h0, j - 2);
            for (uint32_t i = threadIdx.x; i < dw * dh; i += blockDim.x) {
                const int x = (int)(i % dw), y = (int)(i / dw);
                float r;
                if (j == 1)
                    r = reduce_texel(x, y, dw, dh, sw, sh, [&](int sx, int sy) { return depth_at(V.depth_id, w, sx, sy); });
                else
                    r = reduce_texel(x, y, dw, dh, sw, sh,
                                     [&](int sx, int sy) { return __ldcg(src + (size_t)sy * sw + sx); });
                dst[i] = r;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) V.counters[3] = 0;  // ready for the next reduce of this view
}

}  // namespace

uint32_t hiz_tail_floats(uint32_t w, uint32_t h, uint32_t levels) {
    // the levels above the tiled ones that have no zero dimension
    const int top = hiz_tile_levels(w, h, levels);
    uint32_t sum = 0;
    for (uint32_t j = (uint32_t)top + 1; top > 0 && j <= levels && (w >> j) != 0 && (h >> j) != 0; ++j)
        sum += (w >> j) * (h >> j);
    return sum;
}

void launch_hiz(const DeviceView* views, uint32_t nviews, uint32_t tiles_x, uint32_t tiles_y, uint32_t tail,
                uint32_t* status, cudaStream_t stream) {
    // The dynamic shared-memory limit is a per-device function attribute:
    // set it once for each device a launch runs on (setting it twice is
    // harmless, so concurrent first launches need no lock).
    static std::atomic<uint64_t> attr_devices{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (!bit || !(attr_devices.load(std::memory_order_acquire) & bit)) {
        cudaFuncSetAttribute(k_hiz, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailMax * (int)sizeof(float));
        attr_devices.fetch_or(bit, std::memory_order_release);
    }
    // the tail works in shared memory when all of its levels fit
    if (tail > (uint32_t)kTailMax) tail = 0;
    const uint32_t floats = tail > (uint32_t)kTileFloats ? tail : (uint32_t)kTileFloats;
    dim3 grid(tiles_x ? tiles_x : 1, tiles_y ? tiles_y : 1, nviews);
    launch_pdl(k_hiz, grid, dim3(kThreads), floats * sizeof(float), stream, views, status, tail);
}

}  // namespace vkgv
