// Visibility-buffer rasterisation: the mesh shader
// (shaders/visbuffer/visbuffer.mesh.glsl:30-104), the fixed-function
// rasteriser with the pipeline state of application.cpp:326-340 / 830-841, and
// the fragment shader's ID write (shaders/visbuffer/visbuffer.frag.glsl:36).
//
// One warp owns one surviving meshlet draw: it transforms the <= 64 meshlet
// vertices into shared memory, then each lane sets up one triangle at a time
// (homogeneous backface determinant, outcode reject, near/far and guard-band
// clipping, 28.8 fixed-point snap, top-left edge functions, depth plane).
// Small triangles are rasterised by the lane itself; larger ones are cut into
// chunk x chunk pixel rectangles and binned into a queue that a second
// kernel drains with one CTA per rectangle.  Every covered sample performs a
// 64-bit max of (depth bits << 32 | id + 1), which is the order-independent
// form of the GREATER_OR_EQUAL depth test with ties won by the later draw.
#include "kernels.cuh"

namespace vkgv {

namespace {

constexpr float kGuard = 256.0f;
enum : int { OC_XLO = 1, OC_XHI = 2, OC_YLO = 4, OC_YHI = 8, OC_ZLO = 16, OC_ZHI = 32 };

__device__ __forceinline__ int outcode(const float4& v) {
    int c = 0;
    if (v.x < -v.w) c |= OC_XLO;
    if (v.x > v.w) c |= OC_XHI;
    if (v.y < -v.w) c |= OC_YLO;
    if (v.y > v.w) c |= OC_YHI;
    if (v.z < 0.0f) c |= OC_ZLO;
    if (v.z > v.w) c |= OC_ZHI;
    return c;
}

__device__ __forceinline__ bool outside_guard(const float4& v) {
    float g = fmul(kGuard, v.w);
    return v.x < -g || v.x > g || v.y < -g || v.y > g;
}

struct RasterCtx {
    unsigned long long* depth;
    uint32_t w, h;
    float hw, hh;
    uint32_t view;
    BigTri* big;
    uint32_t* big_count;
    uint32_t big_cap;
    uint32_t small_area;
    uint32_t chunk;
    uint32_t* status;
};

// The depth test: a 64-bit max whose result is not needed (a reduction
// that does not wait for the L2 round trip).
__device__ __forceinline__ void plot(unsigned long long* p, unsigned long long v) { atomicMax(p, v); }

__device__ void raster_rect(const int32_t* X, const int32_t* Y, const int32_t* bias, float z0, float pa, float pb,
                            uint32_t id, int px0, int py0, int px1, int py1, unsigned long long* depth,
                            uint32_t w) {
    const unsigned long long lo = (unsigned long long)id + 1ull;
    const int32_t sx0 = px0 * 256 + 128, sy0 = py0 * 256 + 128;
    int64_t erow[3], stx[3], sty[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a = k, b = (k + 1) % 3;
        const int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
        erow[k] = (int64_t)dx * (sy0 - Y[a]) - (int64_t)dy * (sx0 - X[a]);
        stx[k] = -(int64_t)dy * 256;
        sty[k] = (int64_t)dx * 256;
    }
    for (int py = py0; py <= py1; ++py) {
        int64_t e0 = erow[0], e1 = erow[1], e2 = erow[2];
        const int32_t sy = py * 256 + 128;
        const float zrow = __fmaf_rn(pb, __int2float_rn(sy - Y[0]), z0);
        unsigned long long* row = depth + (size_t)py * w;
        for (int px = px0; px <= px1; ++px) {
            if (e0 >= bias[0] && e1 >= bias[1] && e2 >= bias[2]) {
                const int32_t sx = px * 256 + 128;
                float z = __fmaf_rn(pa, __int2float_rn(sx - X[0]), zrow);
                if (!(z > 0.0f)) z = 0.0f;
                if (z > 1.0f) z = 1.0f;
                plot(row + px, ((unsigned long long)__float_as_uint(z) << 32) | lo);
            }
            e0 += stx[0];
            e1 += stx[1];
            e2 += stx[2];
        }
        erow[0] += sty[0];
        erow[1] += sty[1];
        erow[2] += sty[2];
    }
}

// Triangle setup on snapped vertices and dispatch to inline or binned raster.
__device__ __noinline__ void setup_and_raster(int32_t X0, int32_t Y0, float Z0, int32_t X1, int32_t Y1, float Z1, int32_t X2,
                                 int32_t Y2, float Z2, uint32_t id, const RasterCtx& c) {
    int64_t A = (int64_t)(X1 - X0) * (Y2 - Y0) - (int64_t)(Y1 - Y0) * (X2 - X0);
    if (A == 0) return;
    if (A < 0) {
        int32_t tx = X1, ty = Y1;
        float tz = Z1;
        X1 = X2, Y1 = Y2, Z1 = Z2;
        X2 = tx, Y2 = ty, Z2 = tz;
        A = -A;
    }
    const int32_t minx = min(X0, min(X1, X2)), maxx = max(X0, max(X1, X2));
    const int32_t miny = min(Y0, min(Y1, Y2)), maxy = max(Y0, max(Y1, Y2));
    // ceil((min - 128) / 256) and floor((max - 128) / 256); >> is floor division.
    int64_t px0 = ((int64_t)minx - 128 + 255) >> 8, px1 = ((int64_t)maxx - 128) >> 8;
    int64_t py0 = ((int64_t)miny - 128 + 255) >> 8, py1 = ((int64_t)maxy - 128) >> 8;
    px0 = px0 < 0 ? 0 : px0;
    py0 = py0 < 0 ? 0 : py0;
    px1 = px1 > (int64_t)c.w - 1 ? (int64_t)c.w - 1 : px1;
    py1 = py1 > (int64_t)c.h - 1 ? (int64_t)c.h - 1 : py1;
    if (px0 > px1 || py0 > py1) return;
    int32_t X[3] = {X0, X1, X2}, Y[3] = {Y0, Y1, Y2};
    int32_t bias[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a = k, b = (k + 1) % 3;
        const int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
        bias[k] = (dy < 0 || (dy == 0 && dx > 0)) ? 0 : 1;
    }
    const float dx1 = __int2float_rn(X1 - X0), dy1 = __int2float_rn(Y1 - Y0);
    const float dx2 = __int2float_rn(X2 - X0), dy2 = __int2float_rn(Y2 - Y0);
    const float af = __ll2float_rn(A);
    const float dz1 = fsub(Z1, Z0), dz2 = fsub(Z2, Z0);
    const float pa = fdiv(fsub(fmul(dz1, dy2), fmul(dz2, dy1)), af);
    const float pb = fdiv(fsub(fmul(dz2, dx1), fmul(dz1, dx2)), af);
    const int64_t bw = px1 - px0 + 1, bh = py1 - py0 + 1;
    if (bw * bh <= (int64_t)c.small_area) {
        raster_rect(X, Y, bias, Z0, pa, pb, id, (int)px0, (int)py0, (int)px1, (int)py1, c.depth, c.w);
        return;
    }
    const int64_t cs = c.chunk;
    const int64_t ncx = (bw + cs - 1) / cs, ncy = (bh + cs - 1) / cs;
    const uint32_t n = (uint32_t)(ncx * ncy);
    const uint32_t base = atomicAdd(c.big_count, n);
    for (uint32_t i = 0; i < n; ++i) {
        const int64_t cx = i % ncx, cy = i / ncx;
        const int qx0 = (int)(px0 + cx * cs), qy0 = (int)(py0 + cy * cs);
        const int qx1 = (int)min(px1, px0 + (cx + 1) * cs - 1), qy1 = (int)min(py1, py0 + (cy + 1) * cs - 1);
        if (base + i < c.big_cap) {
            BigTri t;
            t.x[0] = X0, t.x[1] = X1, t.x[2] = X2;
            t.y[0] = Y0, t.y[1] = Y1, t.y[2] = Y2;
            t.z0 = Z0, t.pa = pa, t.pb = pb;
            t.id = id;
            t.px0 = (uint16_t)qx0, t.py0 = (uint16_t)qy0, t.px1 = (uint16_t)qx1, t.py1 = (uint16_t)qy1;
            t.view = c.view;
            t._pad = 0;
            c.big[base + i] = t;
        } else {
            report(c.status, kStatusQueueOverflow, base + i);
            raster_rect(X, Y, bias, Z0, pa, pb, id, qx0, qy0, qx1, qy1, c.depth, c.w);
        }
    }
}

__device__ __forceinline__ bool snap(const float4& v, const RasterCtx& c, int32_t& X, int32_t& Y, float& Z) {
    if (!(v.w > 0.0f)) return false;
    const float xd = fdiv(v.x, v.w), yd = fdiv(v.y, v.w), zd = fdiv(v.z, v.w);
    const float xf = fadd(fmul(xd, c.hw), c.hw), yf = fadd(fmul(yd, c.hh), c.hh);
    const float sx = fmul(xf, 256.0f), sy = fmul(yf, 256.0f);
    if (!(fabsf(sx) < 1073741824.0f) || !(fabsf(sy) < 1073741824.0f)) return false;
    X = __float2int_rn(sx);
    Y = __float2int_rn(sy);
    Z = zd;
    return true;
}

__device__ __forceinline__ float plane_dist(const float4& v, int plane) {
    switch (plane) {
        case 0: return fsub(v.w, v.z);
        case 1: return v.z;
        case 2: return fsub(fmul(kGuard, v.w), v.x);
        case 3: return fadd(v.x, fmul(kGuard, v.w));
        case 4: return fsub(fmul(kGuard, v.w), v.y);
        default: return fadd(v.y, fmul(kGuard, v.w));
    }
}

__device__ int clip_poly(const float4* in, int n, float4* out, int plane) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const float4 a = in[i];
        const float4 b = in[(i + 1) % n];
        const float da = plane_dist(a, plane), db = plane_dist(b, plane);
        const bool ia = da >= 0.0f, ib = db >= 0.0f;
        if (ia) out[m++] = a;
        if (ia != ib) {
            const float t = fdiv(da, fsub(da, db));
            out[m++] = make_float4(fadd(a.x, fmul(t, fsub(b.x, a.x))), fadd(a.y, fmul(t, fsub(b.y, a.y))),
                                   fadd(a.z, fmul(t, fsub(b.z, a.z))), fadd(a.w, fmul(t, fsub(b.w, a.w))));
        }
    }
    return m;
}

// Slow path: homogeneous clipping (near/far, then guard band) and a fan.
__device__ __noinline__ void raster_clipped(float4 v0, float4 v1, float4 v2, bool clipz, uint32_t id,
                                            const RasterCtx& c) {
    float4 bufa[12], bufb[12];
    bufa[0] = v0, bufa[1] = v1, bufa[2] = v2;
    float4* cur = bufa;
    float4* nxt = bufb;
    int n = 3;
    if (clipz) {
        for (int plane = 0; plane < 2 && n >= 3; ++plane) {
            n = clip_poly(cur, n, nxt, plane);
            float4* t = cur;
            cur = nxt;
            nxt = t;
        }
    }
    bool guard = false;
    for (int k = 0; k < n; ++k) guard |= outside_guard(cur[k]);
    if (guard) {
        for (int plane = 2; plane < 6 && n >= 3; ++plane) {
            n = clip_poly(cur, n, nxt, plane);
            float4* t = cur;
            cur = nxt;
            nxt = t;
        }
    }
    if (n < 3) return;
    int32_t X[12], Y[12];
    float Z[12];
    for (int k = 0; k < n; ++k)
        if (!snap(cur[k], c, X[k], Y[k], Z[k])) return;
    for (int k = 1; k + 1 < n; ++k)
        setup_and_raster(X[0], Y[0], Z[0], X[k], Y[k], Z[k], X[k + 1], Y[k + 1], Z[k + 1], id, c);
}

struct RasterParams {
    SceneArgs S;
    const DeviceView* views;
    RasterLists lists;
    BigTri* big;
    uint32_t* big_count;
    uint32_t big_cap;
    uint32_t small_area;
    uint32_t chunk;
    uint32_t* status;
};

// Setup record of one small triangle, shared by the warp while it
// rasterises all small triangles of a round cooperatively.
struct TriRec {
    int32_t x[3], y[3];   // oriented (positive area) snapped vertices, 28.8
    float z0, pa, pb;     // depth plane
    float inv_bw;         // 1 / bbox width (exact floor division for bw <= 64)
    uint32_t id;
    uint16_t bx0, by0;    // clamped bbox origin (pixels)
    uint8_t bw, bh;       // clamped bbox extent (pixels, <= 64)
    uint8_t bias;         // bit k: edge k excludes its samples (not top-left)
    uint8_t _pad;
};

constexpr uint8_t kFlagGuard = 1u << 6;
constexpr uint8_t kFlagSnapped = 1u << 7;
// Triangles whose unclamped bbox is below this many 28.8 units on both axes
// keep every edge-function value of their bbox inside int32.
constexpr int32_t kSmallExtent = 1 << 14;

enum TriKind : int { kDrop = 0, kFast = 1, kSlowClip = 2, kSlowSetup = 3 };

#ifndef VKGV_RASTER_WARPS_PER_SM
#define VKGV_RASTER_WARPS_PER_SM 32
#endif

// Warp-per-meshlet raster.  The fast instance (SLOW = false) handles every
// triangle that needs no clipping and fits the cooperative small-triangle
// path, and appends a meshlet that has any other triangle to the view's
// deferred list.  The slow instance (SLOW = true) re-runs those meshlets and
// handles only the remaining triangles (homogeneous clipping, large or
// off-screen-spanning triangles), so the fast instance calls no function.
template <int WARPS, bool SLOW>
__global__ void __launch_bounds__(WARPS * 32, (SLOW ? 16 : VKGV_RASTER_WARPS_PER_SM) / WARPS) k_raster(RasterParams P) {
    __shared__ float4 s_clip[WARPS][64];
    // per vertex: {X, Y (28.8), Z bits, flags} read with one 16-byte load
    __shared__ int4 s_vtx[WARPS][64];
    // the meshlet's triangle-index bytes (<= 126 triangles)
    __shared__ uint32_t s_idx[WARPS][96];
    __shared__ TriRec s_tri[WARPS][32];
    __shared__ uint32_t s_end[WARPS][32];
    __shared__ float s_mvp[WARPS][16];
    __shared__ float s_tdet[WARPS];
    __shared__ float s_vp[16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t vi = blockIdx.y;
    const DeviceView& V = P.views[vi];
    if (threadIdx.x < 16) s_vp[threadIdx.x] = V.cam->view_projection[threadIdx.x];
    __syncthreads();
    const uint32_t slot = P.lists.deferred_slot;
    const uint32_t defer_cap = P.S.draw_count;
    const uint32_t* list;
    uint32_t count, first = 0;
    if (SLOW) {
        list = V.deferred;
        count = min(V.counters[slot], defer_cap);
    } else if (P.lists.pass == 1) {
        list = V.survivors;
        count = min(V.counters[0], V.survivor_capacity);
    } else if (P.lists.pass == 2) {
        const uint32_t c0 = min(V.counters[0], V.survivor_capacity);
        list = V.survivors + c0;
        count = min(V.counters[2], V.survivor_capacity - c0);
    } else {
        list = P.lists.list;
        count = *P.lists.count;
        first = P.lists.first;
    }
    RasterCtx c;
    c.depth = V.depth_id;
    c.w = V.w;
    c.h = V.h;
    c.hw = 0.5f * (float)V.w;
    c.hh = 0.5f * (float)V.h;
    c.view = vi;
    c.big = P.big;
    c.big_count = P.big_count;
    c.big_cap = P.big_cap;
    c.small_area = P.small_area;
    c.chunk = P.chunk;
    c.status = P.status;
    float4* clip = s_clip[warp];
    int4* svtx = s_vtx[warp];
    uint32_t* sidx = s_idx[warp];
    const uint8_t* sidx8 = reinterpret_cast<const uint8_t*>(sidx);
    TriRec* recs = s_tri[warp];
    uint32_t* ends = s_end[warp];
    const uint32_t stride = gridDim.x * WARPS;
    for (uint32_t s = first + blockIdx.x * WARPS + warp; s < count; s += stride) {
        const uint32_t d = list[s];
        if (d >= P.S.draw_count) {
            if (lane == 0) report(P.status, kStatusBadIndex, d);
            continue;
        }
        const vkgv_meshlet_draw dr = P.S.draws[d];
        const vkgv_primitive* prim = &P.S.prims[dr.primitive_index];
        if (dr.meshlet_index >= prim->meshlet_count) {
            if (lane == 0) report(P.status, kStatusBadIndex, d);
            continue;
        }
        const vkgv_meshlet* ml = reinterpret_cast<const vkgv_meshlet*>(prim->meshlet_buffer) + dr.meshlet_index;
        const uint32_t vc = ml->vertex_count, tc = ml->triangle_count;
        if (vc > VKGV_MAX_VERTICES || tc > VKGV_MAX_PRIMITIVES) {
            if (lane == 0) report(P.status, kStatusBadIndex, d);
            continue;
        }
        const uint32_t* vidx = reinterpret_cast<const uint32_t*>(prim->vertex_index_buffer) + ml->vertex_offset;
        const uint8_t* tri = reinterpret_cast<const uint8_t*>(prim->primitive_index_buffer) + ml->triangle_offset;
        const vkgv_vertex* verts = reinterpret_cast<const vkgv_vertex*>(prim->vertex_buffer);
        const bool double_sided = P.S.mats[prim->material_index].double_sided != 0;
        // mvp = VP * M, one element per lane (lanes 0-15); lane 16 takes the
        // sign source determinant(M) of visbuffer.mesh.glsl:71.
        const float* Mg = P.S.transforms + 16 * (size_t)dr.transform_index;
        if (lane < 16) {
            const int cc = lane >> 2, j = lane & 3;
            const float4 mc = __ldg(reinterpret_cast<const float4*>(Mg) + cc);
            s_mvp[warp][lane] = fadd(fadd(fadd(fmul(s_vp[0 * 4 + j], mc.x), fmul(s_vp[1 * 4 + j], mc.y)),
                                          fmul(s_vp[2 * 4 + j], mc.z)),
                                     fmul(s_vp[3 * 4 + j], mc.w));
        } else if (lane == 16) {
            float M[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) M[q] = __ldg(Mg + q);
            s_tdet[warp] = det4(M);
        }
        __syncwarp();
        const float tdet = s_tdet[warp];
        const float* mvp = s_mvp[warp];
        // Vertex stage: clip position, outcode, guard flag and the 28.8 snap,
        // each computed once per meshlet vertex.
        for (uint32_t k = lane; k < vc; k += 32) {
            const vkgv_vertex* vx = verts + __ldg(vidx + k);
            const float2 xy = __ldg(reinterpret_cast<const float2*>(vx->position));
            const float zz = __ldg(&vx->position[2]);
            float r[4];
            m4v(mvp, xy.x, xy.y, zz, 1.0f, r);
            const float4 cv = make_float4(r[0], r[1], r[2], r[3]);
            clip[k] = cv;
            int32_t X = 0, Y = 0;
            float Z = 0.0f;
            uint32_t fl = (uint32_t)outcode(cv);
            if (outside_guard(cv)) fl |= kFlagGuard;
            if (snap(cv, c, X, Y, Z)) fl |= kFlagSnapped;
            svtx[k] = make_int4(X, Y, __float_as_int(Z), (int)fl);
        }
        // Triangle-index bytes into shared memory, 32-bit loads when the
        // block is 4-byte aligned (meshoptimizer pads each block to 4).
        {
            const uint32_t nbytes = 3 * tc;
            if ((reinterpret_cast<uintptr_t>(tri) & 3u) == 0) {
                const uint32_t* tw = reinterpret_cast<const uint32_t*>(tri);
                for (uint32_t k = lane; k < (nbytes + 3) / 4; k += 32) sidx[k] = __ldg(tw + k);
            } else {
                uint8_t* b = reinterpret_cast<uint8_t*>(sidx);
                for (uint32_t k = lane; k < nbytes; k += 32) b[k] = __ldg(tri + k);
            }
        }
        __syncwarp();
        bool any_slow = false;
        for (uint32_t tbase = 0; tbase < tc; tbase += 32) {
            const uint32_t t = tbase + lane;
            uint32_t area = 0;
            if (t < tc) {
                const uint32_t i0 = sidx8[3 * t], i1 = sidx8[3 * t + 1], i2 = sidx8[3 * t + 2];
                const uint32_t id = (d << 7) | t;
                int kind = kDrop;
                int4 q0 = make_int4(0, 0, 0, 0), q1 = q0, q2 = q0;
                int32_t minx = 0, maxx = 0, miny = 0, maxy = 0;
                int64_t A = 0;
                if (i0 >= vc || i1 >= vc || i2 >= vc) {
                    if (!SLOW) report(P.status, kStatusBadIndex, d);
                } else {
                    q0 = svtx[i0], q1 = svtx[i1], q2 = svtx[i2];
                    const uint32_t f0 = (uint32_t)q0.w, f1 = (uint32_t)q1.w, f2 = (uint32_t)q2.w;
                    // The backface test (visbuffer.mesh.glsl:86-101) and the
                    // empty-bbox test are both pure filters, so the cheap
                    // bbox test runs first for triangles that need no clipping.
                    auto backfacing = [&]() {
                        if (double_sided) return false;
                        const float4 a = clip[i0], b = clip[i1], cc = clip[i2];
                        const float det = det3(a.x, a.y, a.w, b.x, b.y, b.w, cc.x, cc.y, cc.w);
                        return tdet < 0.0f ? det < 0.0f : det > 0.0f;
                    };
                    if (f0 & f1 & f2 & 63) {
                        kind = kDrop;  // outcode reject
                    } else if ((f0 | f1 | f2) & (OC_ZLO | OC_ZHI | kFlagGuard)) {
                        kind = backfacing() ? kDrop : kSlowClip;
                    } else if (f0 & f1 & f2 & kFlagSnapped) {
                        minx = min(q0.x, min(q1.x, q2.x)), maxx = max(q0.x, max(q1.x, q2.x));
                        miny = min(q0.y, min(q1.y, q2.y)), maxy = max(q0.y, max(q1.y, q2.y));
                        const int32_t qx0 = max((minx - 128 + 255) >> 8, 0), qx1 = min((maxx - 128) >> 8, (int32_t)c.w - 1);
                        const int32_t qy0 = max((miny - 128 + 255) >> 8, 0), qy1 = min((maxy - 128) >> 8, (int32_t)c.h - 1);
                        if (qx0 <= qx1 && qy0 <= qy1 && !backfacing()) {
                            A = (int64_t)(q1.x - q0.x) * (q2.y - q0.y) - (int64_t)(q1.y - q0.y) * (q2.x - q0.x);
                            if (A != 0) {
                                const bool small = maxx - minx < kSmallExtent && maxy - miny < kSmallExtent &&
                                                   (uint32_t)((qx1 - qx0 + 1) * (qy1 - qy0 + 1)) <= c.small_area;
                                kind = small ? kFast : kSlowSetup;
                            }
                        }
                    }
                }
                if (SLOW) {
                    if (kind == kSlowClip) {
                        raster_clipped(clip[i0], clip[i1], clip[i2],
                                       (((uint32_t)q0.w | (uint32_t)q1.w | (uint32_t)q2.w) & (OC_ZLO | OC_ZHI)) != 0,
                                       id, c);
                    } else if (kind == kSlowSetup) {
                        setup_and_raster(q0.x, q0.y, __int_as_float(q0.z), q1.x, q1.y, __int_as_float(q1.z), q2.x,
                                         q2.y, __int_as_float(q2.z), id, c);
                    }
                } else if (kind == kSlowClip || kind == kSlowSetup) {
                    any_slow = true;
                } else if (kind == kFast) {
                    int2 p0 = make_int2(q0.x, q0.y), p1 = make_int2(q1.x, q1.y), p2 = make_int2(q2.x, q2.y);
                    float z0 = __int_as_float(q0.z), z1 = __int_as_float(q1.z), z2 = __int_as_float(q2.z);
                    if (A < 0) {
                        const int2 tp = p1;
                        p1 = p2;
                        p2 = tp;
                        const float tz = z1;
                        z1 = z2;
                        z2 = tz;
                    }
                    const int64_t Ap = A < 0 ? -A : A;
                    const int32_t px0 = max((minx - 128 + 255) >> 8, 0), px1 = min((maxx - 128) >> 8, (int32_t)c.w - 1);
                    const int32_t py0 = max((miny - 128 + 255) >> 8, 0), py1 = min((maxy - 128) >> 8, (int32_t)c.h - 1);
                    const uint32_t bw = (uint32_t)(px1 - px0 + 1), bh = (uint32_t)(py1 - py0 + 1);
                    TriRec& r = recs[lane];
                    r.x[0] = p0.x, r.x[1] = p1.x, r.x[2] = p2.x;
                    r.y[0] = p0.y, r.y[1] = p1.y, r.y[2] = p2.y;
                    uint8_t bias = 0;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const int32_t dx = r.x[(k + 1) % 3] - r.x[k], dy = r.y[(k + 1) % 3] - r.y[k];
                        if (!(dy < 0 || (dy == 0 && dx > 0))) bias |= (uint8_t)(1u << k);
                    }
                    const float dx1 = __int2float_rn(p1.x - p0.x), dy1 = __int2float_rn(p1.y - p0.y);
                    const float dx2 = __int2float_rn(p2.x - p0.x), dy2 = __int2float_rn(p2.y - p0.y);
                    const float af = __ll2float_rn(Ap);
                    const float dz1 = fsub(z1, z0), dz2 = fsub(z2, z0);
                    r.z0 = z0;
                    r.pa = fdiv(fsub(fmul(dz1, dy2), fmul(dz2, dy1)), af);
                    r.pb = fdiv(fsub(fmul(dz2, dx1), fmul(dz1, dx2)), af);
                    r.inv_bw = 1.0f / (float)bw;
                    r.id = id;
                    r.bx0 = (uint16_t)px0;
                    r.by0 = (uint16_t)py0;
                    r.bw = (uint8_t)bw;
                    r.bh = (uint8_t)bh;
                    r.bias = bias;
                    area = bw * bh;
                }
            }
            if (SLOW) continue;
            // Warp-cooperative raster of this round's small triangles: an
            // inclusive scan of their bbox areas spreads the pixels evenly.
            uint32_t incl = area;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            ends[lane] = incl;
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (uint32_t p = lane; p < total; p += 32) {
                // smallest j with ends[j] > p
                uint32_t j = 0;
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1)
                    if (ends[j + step - 1] <= p) j += step;
                const TriRec& r = recs[j];
                const uint32_t local = p - (ends[j] - (uint32_t)r.bw * r.bh);
                const uint32_t ly = (uint32_t)(((float)local + 0.5f) * r.inv_bw);
                const uint32_t lx = local - ly * r.bw;
                const int32_t sx = (int32_t)(r.bx0 + lx) * 256 + 128;
                const int32_t sy = (int32_t)(r.by0 + ly) * 256 + 128;
                const int32_t e0 = (r.x[1] - r.x[0]) * (sy - r.y[0]) - (r.y[1] - r.y[0]) * (sx - r.x[0]);
                const int32_t e1 = (r.x[2] - r.x[1]) * (sy - r.y[1]) - (r.y[2] - r.y[1]) * (sx - r.x[1]);
                const int32_t e2 = (r.x[0] - r.x[2]) * (sy - r.y[2]) - (r.y[0] - r.y[2]) * (sx - r.x[2]);
                if (e0 >= (int32_t)(r.bias & 1u) && e1 >= (int32_t)((r.bias >> 1) & 1u) &&
                    e2 >= (int32_t)((r.bias >> 2) & 1u)) {
                    float z = __fmaf_rn(r.pa, __int2float_rn(sx - r.x[0]),
                                        __fmaf_rn(r.pb, __int2float_rn(sy - r.y[0]), r.z0));
                    if (!(z > 0.0f)) z = 0.0f;
                    if (z > 1.0f) z = 1.0f;
                    plot(c.depth + (size_t)(r.by0 + ly) * c.w + (r.bx0 + lx),
                         ((unsigned long long)__float_as_uint(z) << 32) | ((unsigned long long)r.id + 1ull));
                }
            }
            __syncwarp();
        }
        if (!SLOW && __any_sync(0xffffffffu, any_slow) && lane == 0) {
            const uint32_t k = atomicAdd(&V.counters[slot], 1u);
            if (k < defer_cap)
                V.deferred[k] = d;
            else
                report(P.status, kStatusListOverflow, d);
        }
        __syncwarp();
    }
}

// Drains the binned rectangles: one CTA per rectangle, its 256 threads laid
// out as chunk x (256 / chunk).
__global__ void __launch_bounds__(256) k_raster_big(const BigTri* __restrict__ q, const uint32_t* count,
                                                    uint32_t cap, const DeviceView* __restrict__ views,
                                                    uint32_t chunk) {
    const uint32_t n = min(*count, cap);
    const int tx = (int)(threadIdx.x % chunk), ty = (int)(threadIdx.x / chunk);
    const int rows = (int)(256 / chunk);
    for (uint32_t e = blockIdx.x; e < n; e += gridDim.x) {
        const BigTri t = q[e];
        const DeviceView& V = views[t.view];
        unsigned long long* depth = V.depth_id;
        const uint32_t w = V.w;
        const unsigned long long lo = (unsigned long long)t.id + 1ull;
        int32_t bias[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int a = k, b = (k + 1) % 3;
            const int32_t dx = t.x[b] - t.x[a], dy = t.y[b] - t.y[a];
            bias[k] = (dy < 0 || (dy == 0 && dx > 0)) ? 0 : 1;
        }
        for (int py = t.py0 + ty; py <= (int)t.py1; py += rows) {
            const int32_t sy = py * 256 + 128;
            const float zrow = __fmaf_rn(t.pb, __int2float_rn(sy - t.y[0]), t.z0);
            for (int px = t.px0 + tx; px <= (int)t.px1; px += (int)chunk) {
                const int32_t sx = px * 256 + 128;
                bool covered = true;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int a = k, b = (k + 1) % 3;
                    const int64_t ev = (int64_t)(t.x[b] - t.x[a]) * (sy - t.y[a]) -
                                       (int64_t)(t.y[b] - t.y[a]) * (sx - t.x[a]);
                    covered = covered && ev >= bias[k];
                }
                if (!covered) continue;
                float z = __fmaf_rn(t.pa, __int2float_rn(sx - t.x[0]), zrow);
                if (!(z > 0.0f)) z = 0.0f;
                if (z > 1.0f) z = 1.0f;
                plot(depth + (size_t)py * w + px, ((unsigned long long)__float_as_uint(z) << 32) | lo);
            }
        }
    }
}

template <int WARPS>
void launch_variant(const RasterParams& P, dim3 grid, cudaStream_t stream) {
    k_raster<WARPS, false><<<grid, WARPS * 32, 0, stream>>>(P);
    k_raster<WARPS, true><<<grid, WARPS * 32, 0, stream>>>(P);
}

}  // namespace

void launch_raster(const SceneArgs& S, const DeviceView* views, uint32_t nviews, const RasterLists& lists,
                   const RasterConfig& cfg, BigTri* big, uint32_t* big_count, uint32_t big_capacity,
                   uint32_t* status, uint32_t sm_count, cudaStream_t stream, cudaEvent_t between) {
    RasterParams P;
    P.S = S;
    P.views = views;
    P.lists = lists;
    P.big = big;
    P.big_count = big_count;
    P.big_cap = big_capacity;
    P.small_area = cfg.small_area;
    P.chunk = cfg.chunk;
    P.status = status;
    uint32_t bpv = cfg.blocks_per_view ? cfg.blocks_per_view : (sm_count * 16 + nviews - 1) / nviews;
    if (bpv == 0) bpv = 1;
    dim3 grid(bpv, nviews);
    switch (cfg.warps_per_cta) {
        case 1: launch_variant<1>(P, grid, stream); break;
        case 2: launch_variant<2>(P, grid, stream); break;
        case 8: launch_variant<8>(P, grid, stream); break;
        default: launch_variant<4>(P, grid, stream); break;
    }
    if (between) cudaEventRecord(between, stream);
    const uint32_t chunk = cfg.chunk >= 8 && cfg.chunk <= 64 ? cfg.chunk : 32;
    k_raster_big<<<sm_count * 8, 256, 0, stream>>>(big, big_count, big_capacity, views, chunk);
}

}  // namespace vkgv
