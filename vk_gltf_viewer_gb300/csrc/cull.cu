// Meshlet culling: the task shader (shaders/visbuffer/visbuffer.task.glsl:25-76)
// as one thread per meshlet draw with warp-ballot compaction.
//
// The reference groups 102 draws per task workgroup and compacts them into a
// uint8 payload with subgroupExclusiveAdd; here every draw is tested once and
// survivors are appended to a per-view uint32 list with one atomic per warp.
// The index clamp at visbuffer.task.glsl:41 re-tests draw 101 of a full
// workgroup in 26 extra lanes and appends it up to 27 times; the duplicates
// produce identical fragments, so the survivor *set* (what this kernel emits,
// each draw once) is the reference's.
#include "kernels.cuh"

namespace vkgv {

namespace {

// Corner table of projectAabb (shaders/culling.h.glsl:32-41) as sign bits,
// three per corner (x, y, z; 1 for -1): (1,-1,-1), (1,1,-1), (-1,1,-1),
// (-1,-1,-1), (1,-1,1), (1,1,1), (-1,-1,1), (-1,1,1).
constexpr uint32_t kCornerSigns = 0x2c2f66;

// Exact floor(log2(m)) clamped to [0, levels-1]; m <= 0 or NaN -> 0,
// +inf -> levels-1.
__device__ __forceinline__ int hiz_level(float m, uint32_t levels) {
    int top = (int)levels - 1;
    if (!(m > 0.0f)) return 0;
    if (isinf(m)) return top;
    int e = (int)((__float_as_uint(m) >> 23) & 0xffu) - 127;  // subnormals give < 0 -> 0
    return e < 0 ? 0 : (e > top ? top : e);
}

// The fine occlusion addition (VKGV_CULL_OCCLUSION_FINE): every pyramid
// texel under the projected box [mn0, mx0] x [mn1, mx1] (level-0 texel
// units, widened by 1/64 texel) at the finest level that is reached from the
// view's depth buffer by exact halvings and holds the box in at most 4 x 4
// texels; occluded when all of them are >= mx2.  No such level (an odd view
// side, or a box too large) leaves the HiZ verdict.  The oracle restates the
// same integer footprint and fp32 products.
// An occluding footprint is reported in *foot: level << 28 | a0 << 16 |
// b0 << 4 | (a1 - a0) << 2 | (b1 - b0).
__device__ __forceinline__ bool fine_occluded(const float* pyr, uint32_t pw0, uint32_t ph0, uint32_t plevels,
                                              uint32_t vw, uint32_t vh, float mn0, float mx0, float mn1, float mx1,
                                              float mx2, uint32_t* foot) {
    if ((vw & 1u) || (vh & 1u) || vw == 0 || vh == 0) return false;
    int top = min(__ffs((int)vw), __ffs((int)vh)) - 2;  // min(ctz) - 1
    top = min(top, (int)plevels - 1);
    const int pw = (int)pw0, ph = (int)ph0;
    int i0 = (int)floorf(fsub(fmul(mn0, (float)pw), 0.015625f)), i1 = (int)floorf(fadd(fmul(mx0, (float)pw), 0.015625f));
    int j0 = (int)floorf(fsub(fmul(mn1, (float)ph), 0.015625f)), j1 = (int)floorf(fadd(fmul(mx1, (float)ph), 0.015625f));
    i0 = min(max(i0, 0), pw - 1);
    i1 = min(max(i1, 0), pw - 1);
    j0 = min(max(j0, 0), ph - 1);
    j1 = min(max(j1, 0), ph - 1);
    for (int l = 0; l <= top; ++l) {
        const int a0 = i0 >> l, a1 = i1 >> l, b0 = j0 >> l, b1 = j1 >> l;
        if (a1 - a0 > 3 || b1 - b0 > 3) continue;
        const uint32_t mw = mip_dim(pw0, (uint32_t)l);
        const float* img = pyr + mip_offset(pw0, ph0, (uint32_t)l);
        for (int y = b0; y <= b1; ++y)
            for (int x = a0; x <= a1; ++x)
                if (__ldg(img + (size_t)y * mw + x) < mx2) return false;
        *foot = ((uint32_t)l << 28) | ((uint32_t)a0 << 16) | ((uint32_t)b0 << 4) | ((uint32_t)(a1 - a0) << 2) |
                (uint32_t)(b1 - b0);
        return true;
    }
    return false;
}

// Repeats a fine footprint (the low word of a fine key) on a pyramid of the
// same shape: occluded iff every texel is >= mx2.
__device__ __forceinline__ bool footprint_occluded(uint32_t foot, float mx2, const float* pyr, uint32_t pw0,
                                                   uint32_t ph0) {
    const uint32_t l = foot >> 28, a0 = (foot >> 16) & 0xfffu, b0 = (foot >> 4) & 0xfffu;
    const uint32_t a1 = a0 + ((foot >> 2) & 3u), b1 = b0 + (foot & 3u);
    const uint32_t mw = mip_dim(pw0, l);
    const float* img = pyr + mip_offset(pw0, ph0, l);
    for (uint32_t y = b0; y <= b1; ++y)
        for (uint32_t x = a0; x <= a1; ++x)
            if (__ldg(img + (size_t)y * mw + x) < mx2) return false;
    return true;
}

struct CullResult {
    bool visible;
    bool occluded;
    unsigned long long sample;  // the HiZ sample of an occlusion test (see pack_sample)
};

// One occlusion verdict as 64 bits, for pass 2 to repeat.
// HiZ key: the nearest AABB depth's bits (high word, sign bit clear), the
// mip level (4 bits), the first footprint texel (12 + 12 bits: mips are at
// most 4096 wide) and whether the footprint also takes the next texel on
// each axis.  A footprint's second texel, when footprint_axis reports one,
// is the next texel or the same one (clamped at the edge), and the MIN of a
// texel with itself is that texel, so the flags record only a distinct next
// texel.  A depth with the sign bit set (negative, -0 or a negative NaN)
// loses to every pyramid depth (all >= +0), as +0 does: it is stored as +0.
// Fine key (a draw the HiZ test kept and the fine test rejected; its depth
// is then > 0): the depth's bits with the sign bit set, and the fine
// footprint of fine_occluded.
__device__ __forceinline__ unsigned long long pack_sample(float maxz, int lvl, int x0, int x1, int nx, int y0, int y1,
                                                          int ny) {
    const uint32_t lo = ((uint32_t)lvl << 28) | ((uint32_t)x0 << 16) | ((uint32_t)y0 << 4) |
                        ((nx == 2 && x1 != x0) ? 2u : 0u) | ((ny == 2 && y1 != y0) ? 1u : 0u);
    uint32_t hi = __float_as_uint(maxz);
    if (hi & 0x80000000u) hi = 0u;
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ unsigned long long pack_fine(float maxz, uint32_t foot) {
    return ((unsigned long long)(__float_as_uint(maxz) | 0x80000000u) << 32) | foot;
}

// Repeats a packed lookup on a pyramid of the same shape: visible iff the
// footprint's MIN depth is below the nearest AABB depth.
__device__ __forceinline__ bool sample_visible(unsigned long long key, const float* pyr, uint32_t pw0, uint32_t ph0) {
    const uint32_t lo = (uint32_t)key;
    const float maxz = __uint_as_float((uint32_t)(key >> 32));
    const uint32_t lvl = lo >> 28, x0 = (lo >> 16) & 0xfffu, y0 = (lo >> 4) & 0xfffu;
    const uint32_t mw = mip_dim(pw0, lvl);
    const float* img = pyr + mip_offset(pw0, ph0, lvl);
    float depth = __ldg(img + (size_t)y0 * mw + x0);
    if (lo & 2u) depth = gmin(depth, __ldg(img + (size_t)y0 * mw + x0 + 1));
    if (lo & 1u) {
        depth = gmin(depth, __ldg(img + (size_t)(y0 + 1) * mw + x0));
        if (lo & 2u) depth = gmin(depth, __ldg(img + (size_t)(y0 + 1) * mw + x0 + 1));
    }
    return depth < maxz;
}

__device__ __forceinline__ CullResult cull_one(const SceneArgs& S, const DeviceView& V, const float* frustum, const float* eye,
                                               const float* occl_vp, const float* pyr, uint32_t pw0,
                                               uint32_t ph0, uint32_t plevels, uint32_t flags, uint32_t d,
                                               bool retest, uint32_t* status) {
    CullResult res{false, false, 0ull};
    const vkgv_meshlet_draw dr = S.draws[d];
    const vkgv_primitive* prim = &S.prims[dr.primitive_index];
    if (dr.meshlet_index >= prim->meshlet_count) {
        report(status, kStatusBadIndex, d);
        return res;
    }
    const vkgv_meshlet* ml = reinterpret_cast<const vkgv_meshlet*>(prim->meshlet_buffer) + dr.meshlet_index;
    const float4* M4 = reinterpret_cast<const float4*>(S.transforms + 16 * (size_t)dr.transform_index);
    float M[16];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float4 q = __ldg(M4 + c);
        M[c * 4 + 0] = q.x;
        M[c * 4 + 1] = q.y;
        M[c * 4 + 2] = q.z;
        M[c * 4 + 3] = q.w;
    }
    const float e0 = ml->aabb_extents[0], e1 = ml->aabb_extents[1], e2 = ml->aabb_extents[2];
    float wc4[4];
    // worldAabbCenter (visbuffer.task.glsl:50)
    m4v(M, ml->aabb_center[0], ml->aabb_center[1], ml->aabb_center[2], 1.0f, wc4);
    // getWorldSpaceAabbExtent (culling.h.glsl:22-29)
    float we[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
        we[j] = fadd(fadd(fmul(fabsf(M[0 * 4 + j]), e0), fmul(fabsf(M[1 * 4 + j]), e1)), fmul(fabsf(M[2 * 4 + j]), e2));
    // isAabbInFrustum (culling.h.glsl:8-19).  A pass-2 candidate passed the
    // frustum and cone tests in pass 1 with the same planes and eye, and
    // would pass them again bit for bit, so only its occlusion is re-tested.
    if ((flags & VKGV_CULL_FRUSTUM) && !retest) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float p0 = frustum[4 * i], p1 = frustum[4 * i + 1], p2 = frustum[4 * i + 2], p3 = frustum[4 * i + 3];
            float radius = fadd(fadd(fmul(we[0], fabsf(p0)), fmul(we[1], fabsf(p1))), fmul(we[2], fabsf(p2)));
            float distance = fsub(fadd(fadd(fmul(p0, wc4[0]), fmul(p1, wc4[1])), fmul(p2, wc4[2])), p3);
            if (-radius > distance) return res;
        }
    }
    // Meshlet normal-cone backface test (an addition; conservative with
    // respect to the per-triangle test of visbuffer.mesh.glsl:86-101, which
    // a double-sided material skips).
    if (!retest && eye && S.cone_table && dr.primitive_index < S.primitive_count &&
        !S.mats[prim->material_index].double_sided) {
        const uint64_t cones = S.cone_table[dr.primitive_index];
        if (cones) {
            const vkgv_meshlet_cone& cone = reinterpret_cast<const vkgv_meshlet_cone*>(cones)[dr.meshlet_index];
            bool culled;
            if (V.eyes && dr.transform_index < S.transform_count) {
                const float4 o = __ldg(V.eyes + dr.transform_index);
                culled = o.w != 0.0f && cone_culled_at(cone, o.x, o.y, o.z);
            } else {
                culled = cone_culled(cone, M, eye);
            }
            if (culled) return res;
        }
    }
    if (!pyr) {
        res.visible = true;
        return res;
    }
    // projectAabb (culling.h.glsl:44-56).  Corner i is (wc +- we) per axis
    // (the table's +-1 factors are exact), so each row j of occl_vp * corner,
    // ((m0j x + m1j y) + m2j z) + m3j, is assembled from the two values of
    // m0j x, m1j y and m2j z: the same rounded operations as transforming
    // each corner, with the shared products and partial sums formed once.
    const float ax[2] = {fadd(we[0], wc4[0]), fadd(-we[0], wc4[0])};
    const float ay[2] = {fadd(we[1], wc4[1]), fadd(-we[1], wc4[1])};
    const float az[2] = {fadd(we[2], wc4[2]), fadd(-we[2], wc4[2])};
    float rows[4][2][2][2];  // [j][x sign][y sign][z sign]
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float mx[2] = {fmul(occl_vp[0 * 4 + j], ax[0]), fmul(occl_vp[0 * 4 + j], ax[1])};
        const float my[2] = {fmul(occl_vp[1 * 4 + j], ay[0]), fmul(occl_vp[1 * 4 + j], ay[1])};
        const float mz[2] = {fmul(occl_vp[2 * 4 + j], az[0]), fmul(occl_vp[2 * 4 + j], az[1])};
        const float m3 = fmul(occl_vp[3 * 4 + j], 1.0f);
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const float xy = fadd(mx[a], my[b]);
#pragma unroll
                for (int c = 0; c < 2; ++c) rows[j][a][b][c] = fadd(fadd(xy, mz[c]), m3);
            }
    }
    float mn0 = 1.0f, mn1 = 1.0f, mn2 = 1.0f, mx0 = -1.0f, mx1 = -1.0f, mx2 = -1.0f;
    bool all_front = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t sg = (kCornerSigns >> (3 * i)) & 7u;
        const int a = (int)(sg & 1u), b = (int)((sg >> 1) & 1u), c = (int)(sg >> 2);
        const float clip[4] = {rows[0][a][b][c], rows[1][a][b][c], rows[2][a][b][c], rows[3][a][b][c]};
        all_front &= clip[3] > 0.0f;
        // clip.xyz / clip.w as one correctly rounded reciprocal of w and three
        // products (within GLSL's 2.5 ulp for a division)
        const float rw = __frcp_rn(clip[3]);
        float ndx = gclamp(fmul(clip[0], rw), -1.0f, 1.0f);
        float ndy = gclamp(fmul(clip[1], rw), -1.0f, 1.0f);
        float qx = fadd(fmul(ndx, 0.5f), 0.5f), qy = fadd(fmul(ndy, 0.5f), 0.5f);
        float qz = fmul(clip[2], rw);
        mn0 = gmin(mn0, qx);
        mn1 = gmin(mn1, qy);
        mn2 = gmin(mn2, qz);
        mx0 = gmax(mx0, qx);
        mx1 = gmax(mx1, qy);
        mx2 = gmax(mx2, qz);
    }
    (void)mn2;
    // HiZ lookup (visbuffer.task.glsl:57-64)
    float width = fmul(fsub(mx0, mn0), (float)pw0);
    float height = fmul(fsub(mx1, mn1), (float)ph0);
    int lvl = hiz_level(gmax(width, height), plevels);
    float cx = fmul(fadd(mn0, mx0), 0.5f), cy = fmul(fadd(mn1, mx1), 0.5f);
    uint32_t mw = mip_dim(pw0, (uint32_t)lvl), mh = mip_dim(ph0, (uint32_t)lvl);
    const float* img = pyr + mip_offset(pw0, ph0, (uint32_t)lvl);
    int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
    int nx = footprint_axis(cx, mw, x0, x1);
    int ny = footprint_axis(cy, mh, y0, y1);
    float depth = __ldg(img + (size_t)y0 * mw + x0);
    if (nx == 2) depth = gmin(depth, __ldg(img + (size_t)y0 * mw + x1));
    if (ny == 2) {
        depth = gmin(depth, __ldg(img + (size_t)y1 * mw + x0));
        if (nx == 2) depth = gmin(depth, __ldg(img + (size_t)y1 * mw + x1));
    }
    uint32_t foot = 0;
    if (!(depth < mx2)) {
        res.occluded = true;
        res.sample = pack_sample(mx2, lvl, x0, x1, nx, y0, y1, ny);
    } else if ((flags & VKGV_CULL_OCCLUSION_FINE) && all_front &&
               fine_occluded(pyr, pw0, ph0, plevels, V.w, V.h, mn0, mx0, mn1, mx1, mx2, &foot)) {
        res.occluded = true;
        res.sample = pack_fine(mx2, foot);
    } else {
        res.visible = true;
    }
    return res;
}

// Appends `flag` lanes' values to list[*counter ...] with one atomic per warp.
__device__ __forceinline__ void warp_append(bool flag, uint32_t value, uint32_t* list, uint32_t* counter,
                                            uint32_t capacity, uint32_t* status) {
    const unsigned mask = __ballot_sync(0xffffffffu, flag);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (flag) {
        uint32_t slot = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
        if (slot < capacity)
            list[slot] = value;
        else
            report(status, kStatusListOverflow, slot);
    }
}

// warp_append of a value and its packed HiZ sample into parallel arrays
// (the sample array may be null).
__device__ __forceinline__ void warp_append2(bool flag, uint32_t value, unsigned long long sample, uint32_t* list,
                                             unsigned long long* samples, uint32_t* counter, uint32_t capacity,
                                             uint32_t* status) {
    const unsigned mask = __ballot_sync(0xffffffffu, flag);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (flag) {
        uint32_t slot = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
        if (slot < capacity) {
            list[slot] = value;
            if (samples) samples[slot] = sample;
        } else {
            report(status, kStatusListOverflow, slot);
        }
    }
}

// pass 1: candidates are all draws [0, D); survivors -> survivors[0..),
//         occlusion rejects -> rejected.
// pass 2: candidates are rejected[0, counters[1]); survivors are appended at
//         survivors[counters[0] + ...] via counters[2].
__global__ void __launch_bounds__(256, 5) k_cull(SceneArgs S, const DeviceView* __restrict__ views, uint32_t flags,
                                              uint32_t pass, uint32_t* status) {
    pdl_begin();
    const DeviceView& V = views[blockIdx.y];
    const vkgv_camera* cam = V.cam;
    __shared__ float s_frustum[24];
    __shared__ float s_vp[16];
    __shared__ float s_eye[3];
    __shared__ int s_eye_ok;
    __shared__ int s_same;
    if (threadIdx.x < 24) s_frustum[threadIdx.x] = (&cam->frustum[0][0])[threadIdx.x];
    if (threadIdx.x < 16)
        s_vp[threadIdx.x] = pass == 1 ? cam->prev_occlusion_view_projection[threadIdx.x]
                                      : cam->occlusion_view_projection[threadIdx.x];
    if (threadIdx.x == 32) {
        // the eye of the raster view-projection, for the cone test
        float vp[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) vp[k] = cam->view_projection[k];
        s_eye_ok = (flags & VKGV_CULL_CONE) && S.cone_table && eye_from_vp(vp, s_eye);
    }
    if (threadIdx.x == 64) {
        // Pass 2 can repeat the pass-1 lookups when the occlusion camera and
        // the pyramid's shape are unchanged (a static camera): the same box
        // projects to the same footprint.
        int same = pass == 2 && V.reject_samples != nullptr && V.prev_pyr != nullptr && V.prev_levels != 0 &&
                   V.prev_w0 == (V.w >> 1) && V.prev_h0 == (V.h >> 1) && V.prev_levels == V.pyr_levels;
        for (int k = 0; same && k < 16; ++k)
            same = __float_as_uint(cam->prev_occlusion_view_projection[k]) ==
                   __float_as_uint(cam->occlusion_view_projection[k]);
        s_same = same;
    }
    __syncthreads();
    const float* eye = s_eye_ok ? s_eye : nullptr;
    const float* pyr = nullptr;
    uint32_t pw0 = 0, ph0 = 0, pl = 0;
    if (flags & VKGV_CULL_OCCLUSION) {
        if (pass == 1 && V.prev_pyr && V.prev_levels) {
            pyr = V.prev_pyr;
            pw0 = V.prev_w0;
            ph0 = V.prev_h0;
            pl = V.prev_levels;
        } else if (pass == 2 && V.pyr && V.pyr_levels) {
            pyr = V.pyr;
            pw0 = V.w >> 1;
            ph0 = V.h >> 1;
            pl = V.pyr_levels;
        }
    }
    const bool collect_rejects = pass == 1 && pyr != nullptr && (flags & VKGV_CULL_TWO_PASS);
    const uint32_t n = pass == 1 ? S.draw_count : V.counters[1];
    uint32_t* out_counter = pass == 1 ? &V.counters[0] : &V.counters[2];
    uint32_t* out_list = pass == 1 ? V.survivors : V.survivors + V.counters[0];
    const uint32_t cap = pass == 1 ? V.survivor_capacity : V.survivor_capacity - min(V.counters[0], V.survivor_capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    // Grid-stride with a warp-uniform trip count so the ballots stay converged.
    const uint32_t start = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t warp_start = start & ~31u;
    const bool repeat = s_same != 0 && pyr != nullptr;
    for (uint32_t base = warp_start; base < n; base += stride) {
        const uint32_t i = base + (threadIdx.x & 31);
        bool vis = false, occ = false;
        unsigned long long sample = 0ull;
        uint32_t d = 0;
        if (i < n) {
            d = pass == 1 ? i : V.rejected[i];
            if (d >= S.draw_count) {
                report(status, kStatusBadIndex, d);
            } else {
                // The repeated lookup when it applies: a fine key that still
                // occludes, or a HiZ key that still occludes (or, without
                // the fine test, still keeps), decides; otherwise the full
                // test (which needs the box) runs.
                int verdict = -1;
                if (repeat) {
                    const unsigned long long key = V.reject_samples[i];
                    if (key >> 63) {
                        const float mz = __uint_as_float((uint32_t)(key >> 32) & 0x7fffffffu);
                        if (footprint_occluded((uint32_t)key, mz, pyr, pw0, ph0)) verdict = 0;
                    } else {
                        const bool coarse = sample_visible(key, pyr, pw0, ph0);
                        if (!coarse) verdict = 0;
                        else if (!(flags & VKGV_CULL_OCCLUSION_FINE)) verdict = 1;
                    }
                }
                if (verdict >= 0) {
                    vis = verdict == 1;
                } else {
                    CullResult r = cull_one(S, V, s_frustum, eye, s_vp, pyr, pw0, ph0, pl, flags, d, pass == 2,
                                            status);
                    vis = r.visible;
                    occ = r.occluded;
                    sample = r.sample;
                }
            }
        }
        warp_append(vis, d, out_list, out_counter, cap, status);
        if (collect_rejects)
            warp_append2(occ, d, sample, V.rejected, V.reject_samples, &V.counters[1], S.draw_count, status);
    }
}

}  // namespace

void launch_cull(const SceneArgs& S, const DeviceView* views, uint32_t nviews, uint32_t flags, uint32_t pass,
                 uint32_t* status, uint32_t sm_count, cudaStream_t stream) {
    const uint32_t threads = 256;
    const uint32_t want = (S.draw_count + threads - 1) / threads;
    // Both passes stride over their candidates (pass 1: every draw; pass 2:
    // the reject list, whose length lives on the device) with at most about
    // sm_count * f CTAs over all views: a CTA's prologue (frustum planes,
    // occlusion view-projection, the raster eye from an inverse, in one
    // thread before a barrier) is then paid once per many draws.  256-view
    // batch: pass 1 7.46 -> 5.96 ms, pass 2 1.40 -> 1.19 ms.  A single view
    // takes f = 16 in pass 1 (843,776 draws: 2,432 CTAs instead of one
    // 256-draw CTA per draw block, cull 36 -> 35 us; 8 and 32 were no
    // faster) and f = 8 for its short pass-2 list.
    const uint32_t f = pass == 1 ? (nviews == 1 ? 16u : 128u) : (nviews == 1 ? 8u : 40u);
    const uint32_t fill = (sm_count * f + nviews - 1) / nviews;
    uint32_t per_view = want < fill ? want : fill;
    if (per_view > 65535u) per_view = 65535u;
    if (per_view == 0) per_view = 1;
    dim3 grid(per_view, nviews);
    launch_pdl(k_cull, grid, dim3(threads), 0, stream, S, views, flags, pass, status);
}

}  // namespace vkgv
