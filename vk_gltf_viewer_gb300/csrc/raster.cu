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
// kernel drains with one warp per rectangle.  Every covered sample performs a
// 64-bit max of (depth bits << 32 | id + 1), which is the order-independent
// form of the GREATER_OR_EQUAL depth test with ties won by the later draw.
#include <atomic>

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

// A large triangle of the slow instance, set up and waiting for its binned
// rectangles to be queued: the lanes of a warp collect their jobs while they
// diverge over clipping and setup, then queue all of them with one atomic
// per warp.  (One atomic per triangle on the shared queue counter
// serialised: 23,700 slow triangles in one single-view frame.)
struct BinJob {
    int32_t x[3], y[3];       // oriented snapped vertices, 28.8
    float z0, pa, pb;         // depth plane
    uint32_t id;
    int32_t px0, py0, px1, py1;  // clamped pixel bounding box
    uint32_t n;               // rectangles of c.chunk x c.chunk pixels
};
// A clipped triangle fans into at most 10 triangles.
constexpr uint32_t kMaxJobs = 10;
struct JobList {
    BinJob job[kMaxJobs];
    uint32_t count;
};

// The rectangles of one job, queued at c.big[at, at + n) (past the queue's
// capacity they are drawn in place and the overflow is reported).
__device__ void queue_job(const BinJob& j, uint32_t at, const RasterCtx& c) {
    const int64_t cs = c.chunk;
    const int64_t ncx = ((int64_t)(j.px1 - j.px0 + 1) + cs - 1) / cs;
    for (uint32_t i = 0; i < j.n; ++i, ++at) {
        const int64_t cx = i % ncx, cy = i / ncx;
        const int qx0 = (int)(j.px0 + cx * cs), qy0 = (int)(j.py0 + cy * cs);
        const int qx1 = (int)min((int64_t)j.px1, j.px0 + (cx + 1) * cs - 1);
        const int qy1 = (int)min((int64_t)j.py1, j.py0 + (cy + 1) * cs - 1);
        if (at < c.big_cap) {
            BigTri t;
            t.x[0] = j.x[0], t.x[1] = j.x[1], t.x[2] = j.x[2];
            t.y[0] = j.y[0], t.y[1] = j.y[1], t.y[2] = j.y[2];
            t.z0 = j.z0, t.pa = j.pa, t.pb = j.pb;
            t.id = j.id;
            t.px0 = (uint16_t)qx0, t.py0 = (uint16_t)qy0, t.px1 = (uint16_t)qx1, t.py1 = (uint16_t)qy1;
            t.view = c.view;
            t._pad = 0;
            c.big[at] = t;
        } else {
            report(c.status, kStatusQueueOverflow, at);
            int32_t bias[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int32_t dx = j.x[(k + 1) % 3] - j.x[k], dy = j.y[(k + 1) % 3] - j.y[k];
                bias[k] = (dy < 0 || (dy == 0 && dx > 0)) ? 0 : 1;
            }
            raster_rect(j.x, j.y, bias, j.z0, j.pa, j.pb, j.id, qx0, qy0, qx1, qy1, c.depth, c.w);
        }
    }
}

// Queues the jobs of every lane (the whole warp, converged): an exclusive
// scan of the lanes' rectangle counts, one atomic on the queue counter.
__device__ void flush_jobs(JobList& jobs, const RasterCtx& c, int lane) {
    uint32_t mine = 0;
    for (uint32_t i = 0; i < jobs.count; ++i) mine += jobs.job[i].n;
    uint32_t incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) {
        jobs.count = 0;
        return;
    }
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(c.big_count, total);
    base = __shfl_sync(0xffffffffu, base, 0) + (incl - mine);
    for (uint32_t i = 0; i < jobs.count; ++i) {
        queue_job(jobs.job[i], base, c);
        base += jobs.job[i].n;
    }
    jobs.count = 0;
}

// Triangle setup on snapped vertices and dispatch to inline or binned
// raster; a triangle to bin becomes a job in `jobs` (queued directly when
// the list is full).
__device__ __noinline__ void setup_and_raster(int32_t X0, int32_t Y0, float Z0, int32_t X1, int32_t Y1, float Z1, int32_t X2,
                                 int32_t Y2, float Z2, uint32_t id, const RasterCtx& c, JobList& jobs) {
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
    const float ra = __frcp_rn(af);
    const float pa = fmul(fsub(fmul(dz1, dy2), fmul(dz2, dy1)), ra);
    const float pb = fmul(fsub(fmul(dz2, dx1), fmul(dz1, dx2)), ra);
    const int64_t bw = px1 - px0 + 1, bh = py1 - py0 + 1;
    if (bw * bh <= (int64_t)c.small_area) {
        raster_rect(X, Y, bias, Z0, pa, pb, id, (int)px0, (int)py0, (int)px1, (int)py1, c.depth, c.w);
        return;
    }
    const int64_t cs = c.chunk;
    const int64_t ncx = (bw + cs - 1) / cs, ncy = (bh + cs - 1) / cs;
    BinJob j;
    j.x[0] = X0, j.x[1] = X1, j.x[2] = X2;
    j.y[0] = Y0, j.y[1] = Y1, j.y[2] = Y2;
    j.z0 = Z0, j.pa = pa, j.pb = pb;
    j.id = id;
    j.px0 = (int32_t)px0, j.py0 = (int32_t)py0, j.px1 = (int32_t)px1, j.py1 = (int32_t)py1;
    j.n = (uint32_t)(ncx * ncy);
    if (jobs.count < kMaxJobs) {
        jobs.job[jobs.count++] = j;
    } else {
        queue_job(j, atomicAdd(c.big_count, j.n), c);
    }
}

__device__ __forceinline__ bool snap(const float4& v, const RasterCtx& c, int32_t& X, int32_t& Y, float& Z) {
    if (!(v.w > 0.0f)) return false;
    // one correctly rounded reciprocal of w and three products
    const float rw = __frcp_rn(v.w);
    const float xd = fmul(v.x, rw), yd = fmul(v.y, rw), zd = fmul(v.z, rw);
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
                                            const RasterCtx& c, JobList& jobs) {
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
        setup_and_raster(X[0], Y[0], Z[0], X[k], Y[k], Z[k], X[k + 1], Y[k + 1], Z[k + 1], id, c, jobs);
}

// Views per raster launch (the launcher splits larger batches).
constexpr uint32_t kRasterMaxViews = 1024;

// What the per-meshlet header chain resolves for one work item.
struct ItemHeader {
    const uint32_t* vidx;       // the meshlet's vertex indices
    const uint8_t* tri;         // its triangle-index bytes
    const vkgv_vertex* verts;   // the primitive's vertex stream
    uint32_t d;                 // meshlet draw index
    uint32_t v;                 // view (in this launch)
    uint32_t transform;         // node transform index
    uint8_t vc, tc;             // vertex and triangle counts
    uint8_t double_sided;       // material flag
    uint8_t bad;                // an index out of range: reported, skipped
};

struct RasterParams {
    SceneArgs S;
    const DeviceView* views;  // this launch's views
    uint32_t nviews;          // <= kRasterMaxViews
    uint32_t view_base;       // index of views[0] in the frame's view table
    RasterLists lists;
    BigTri* big;
    uint32_t* big_count;
    uint32_t big_cap;
    uint32_t small_area;
    uint32_t chunk;
    uint32_t* status;
    uint32_t* work;           // [0] items taken, [1] warps done (zero between launches)
};

// The meshlet list a raster instance draws for one view: pass-1 or pass-2
// survivors, the view's deferred meshlets (slow instance), or an explicit
// list; items are list[first, first + count).
template <bool SLOW>
__device__ __forceinline__ void view_work(const RasterParams& P, const DeviceView& V, const uint32_t*& list,
                                          uint32_t& count, uint32_t& first) {
    first = 0;
    if (SLOW) {
        list = V.deferred;
        count = min(V.counters[P.lists.deferred_slot], P.S.draw_count);
    } else if (P.lists.pass == 1) {
        list = V.survivors;
        count = min(V.counters[0], V.survivor_capacity);
    } else if (P.lists.pass == 2) {
        const uint32_t c0 = min(V.counters[0], V.survivor_capacity);
        list = V.survivors + c0;
        count = min(V.counters[2], V.survivor_capacity - c0);
    } else {
        list = P.lists.list;
        const uint32_t n = *P.lists.count;
        first = P.lists.first;
        count = n > first ? n - first : 0u;
    }
}

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
#define VKGV_RASTER_WARPS_PER_SM 28
#endif

// Small triangles whose clamped bbox has at most this many pixels are
// rasterised by their own lane; larger small ones by the whole warp.
#ifndef VKGV_RASTER_LANE_AREA
#define VKGV_RASTER_LANE_AREA 4
#endif
constexpr uint32_t kLaneArea = VKGV_RASTER_LANE_AREA;
// Small triangles above this bbox area are queued for k_raster_big.
#ifndef VKGV_RASTER_QUEUE_AREA
#define VKGV_RASTER_QUEUE_AREA 16
#endif
constexpr uint32_t kQueueArea = VKGV_RASTER_QUEUE_AREA;

struct TriClass {
    int4 q0, q1, q2;  // snapped vertex records {X, Y, Z bits, flags}
};

// Sorts one meshlet triangle into drop / fast / slow-clip / slow-setup.  The
// backface test (visbuffer.mesh.glsl:86-101) and the empty-bbox test are
// both pure filters, so the cheap bbox test runs first for triangles that
// need no clipping.  kFast: snapped, inside the guard band, front-facing,
// non-zero area, a pixel centre in its bbox, bbox within small_area pixels
// and edge values within int32.
template <bool SLOW>
__device__ __forceinline__ int classify(uint32_t i0, uint32_t i1, uint32_t i2, uint32_t vc, const int4* svtx,
                                        const float4* clip, bool double_sided, float tdet, const RasterCtx& c,
                                        uint32_t d, TriClass& k) {
    if (i0 >= vc || i1 >= vc || i2 >= vc) {
        if (!SLOW) report(c.status, kStatusBadIndex, d);
        return kDrop;
    }
    k.q0 = svtx[i0];
    k.q1 = svtx[i1];
    k.q2 = svtx[i2];
    const uint32_t f0 = (uint32_t)k.q0.w, f1 = (uint32_t)k.q1.w, f2 = (uint32_t)k.q2.w;
    auto backfacing = [&]() {
        if (double_sided) return false;
        const float4 a = clip[i0], b = clip[i1], cc = clip[i2];
        const float det = det3(a.x, a.y, a.w, b.x, b.y, b.w, cc.x, cc.y, cc.w);
        return tdet < 0.0f ? det < 0.0f : det > 0.0f;
    };
    if (f0 & f1 & f2 & 63) return kDrop;  // outcode reject
    if ((f0 | f1 | f2) & (OC_ZLO | OC_ZHI | kFlagGuard)) return backfacing() ? kDrop : kSlowClip;
    if (!(f0 & f1 & f2 & kFlagSnapped)) return kDrop;
    const int4 &q0 = k.q0, &q1 = k.q1, &q2 = k.q2;
    const int32_t minx = min(q0.x, min(q1.x, q2.x)), maxx = max(q0.x, max(q1.x, q2.x));
    const int32_t miny = min(q0.y, min(q1.y, q2.y)), maxy = max(q0.y, max(q1.y, q2.y));
    const int32_t qx0 = max((minx - 128 + 255) >> 8, 0), qx1 = min((maxx - 128) >> 8, (int32_t)c.w - 1);
    const int32_t qy0 = max((miny - 128 + 255) >> 8, 0), qy1 = min((maxy - 128) >> 8, (int32_t)c.h - 1);
    if (qx0 > qx1 || qy0 > qy1 || backfacing()) return kDrop;
    const int64_t A = (int64_t)(q1.x - q0.x) * (q2.y - q0.y) - (int64_t)(q1.y - q0.y) * (q2.x - q0.x);
    if (A == 0) return kDrop;
    const bool small = maxx - minx < kSmallExtent && maxy - miny < kSmallExtent &&
                       (uint32_t)((qx1 - qx0 + 1) * (qy1 - qy0 + 1)) <= c.small_area;
    return small ? kFast : kSlowSetup;
}

// First stage of the fast instance, on every triangle: 0 = dropped (an
// index out of range, outcode reject, unsnapped vertex, or no pixel centre
// in its clamped bounding box), 2 = needs the slow instance (a vertex
// outside the near/far planes or the guard band), 1 = a candidate for the
// compacted second stage (raster_small), which applies the backface test
// (visbuffer.mesh.glsl:86-101), the zero-area test and the size limits.
// The tests only filter, so their order does not change what is drawn; the
// cheap ones run here on every triangle, the others only on the candidates.
__device__ __forceinline__ int prefilter(uint32_t i0, uint32_t i1, uint32_t i2, uint32_t vc, const int4* svtx,
                                         const RasterCtx& c, uint32_t d) {
    if (i0 >= vc || i1 >= vc || i2 >= vc) {
        report(c.status, kStatusBadIndex, d);
        return 0;
    }
    const int4 q0 = svtx[i0], q1 = svtx[i1], q2 = svtx[i2];
    const uint32_t f0 = (uint32_t)q0.w, f1 = (uint32_t)q1.w, f2 = (uint32_t)q2.w;
    if (f0 & f1 & f2 & 63) return 0;  // outcode reject
    if ((f0 | f1 | f2) & (OC_ZLO | OC_ZHI | kFlagGuard)) return 2;
    if (!(f0 & f1 & f2 & kFlagSnapped)) return 0;
    const int32_t minx = min(q0.x, min(q1.x, q2.x)), maxx = max(q0.x, max(q1.x, q2.x));
    const int32_t miny = min(q0.y, min(q1.y, q2.y)), maxy = max(q0.y, max(q1.y, q2.y));
    const int32_t qx0 = max((minx - 128 + 255) >> 8, 0), qx1 = min((maxx - 128) >> 8, (int32_t)c.w - 1);
    const int32_t qy0 = max((miny - 128 + 255) >> 8, 0), qy1 = min((maxy - 128) >> 8, (int32_t)c.h - 1);
    return (qx0 > qx1 || qy0 > qy1) ? 0 : 1;
}

// One sample of a small triangle: int32 edge functions (the extent bound of
// kFast keeps them exact), top-left bias, plane depth clamped to [0, 1].
__device__ __forceinline__ void small_sample(const int32_t* x, const int32_t* y, uint32_t bias, float z0, float pa,
                                             float pb, int32_t px, int32_t py, unsigned long long lo,
                                             const RasterCtx& c) {
    const int32_t sx = px * 256 + 128, sy = py * 256 + 128;
    const int32_t e0 = (x[1] - x[0]) * (sy - y[0]) - (y[1] - y[0]) * (sx - x[0]);
    const int32_t e1 = (x[2] - x[1]) * (sy - y[1]) - (y[2] - y[1]) * (sx - x[1]);
    const int32_t e2 = (x[0] - x[2]) * (sy - y[2]) - (y[0] - y[2]) * (sx - x[2]);
    if (e0 >= (int32_t)(bias & 1u) && e1 >= (int32_t)((bias >> 1) & 1u) && e2 >= (int32_t)((bias >> 2) & 1u)) {
        float z = __fmaf_rn(pa, __int2float_rn(sx - x[0]), __fmaf_rn(pb, __int2float_rn(sy - y[0]), z0));
        if (!(z > 0.0f)) z = 0.0f;
        if (z > 1.0f) z = 1.0f;
        plot(c.depth + (size_t)py * c.w + px, ((unsigned long long)__float_as_uint(z) << 32) | lo);
    }
}

// Second stage of the fast instance: up to 32 compacted candidates, one
// per lane (ct = meshlet-local triangle index, 0xffffffff = none).  A
// candidate that is back-facing or of zero area is dropped; one whose bbox
// exceeds small_area pixels or whose extent leaves int32 edge values needs
// the slow instance (the return value); the rest are set up and
// rasterised.  A triangle whose
// clamped bbox has at most kLaneArea pixels is rasterised by its own lane;
// the larger ones are spread over the warp by an inclusive scan of their
// bbox areas.
__device__ __forceinline__ bool raster_small(uint32_t ct, const uint8_t* sidx8, const int4* svtx, const float4* clip,
                                             bool double_sided, float tdet, uint32_t d, const RasterCtx& c,
                                             TriRec* recs, uint32_t* ends, int lane) {
    uint32_t coop_area = 0;
    bool slow = false;
    int4 q0, q1, q2;
    int32_t A = 0;  // the area of a live (small) triangle fits int32
    int32_t px0 = 0, px1 = 0, py0 = 0, py1 = 0;
    bool live = false;
    if (ct != 0xffffffffu) {
        const uint32_t i0 = sidx8[3 * ct], i1 = sidx8[3 * ct + 1], i2 = sidx8[3 * ct + 2];
        q0 = svtx[i0], q1 = svtx[i1], q2 = svtx[i2];
        bool back = false;
        if (!double_sided) {
            const float4 a = clip[i0], b = clip[i1], cc = clip[i2];
            const float det = det3(a.x, a.y, a.w, b.x, b.y, b.w, cc.x, cc.y, cc.w);
            back = tdet < 0.0f ? det < 0.0f : det > 0.0f;
        }
        if (!back) {
            const int32_t minx = min(q0.x, min(q1.x, q2.x)), maxx = max(q0.x, max(q1.x, q2.x));
            const int32_t miny = min(q0.y, min(q1.y, q2.y)), maxy = max(q0.y, max(q1.y, q2.y));
            if (maxx - minx < kSmallExtent && maxy - miny < kSmallExtent) {
                // edge values of such a triangle stay inside int32
                A = (q1.x - q0.x) * (q2.y - q0.y) - (q1.y - q0.y) * (q2.x - q0.x);
                px0 = max((minx - 128 + 255) >> 8, 0), px1 = min((maxx - 128) >> 8, (int32_t)c.w - 1);
                py0 = max((miny - 128 + 255) >> 8, 0), py1 = min((maxy - 128) >> 8, (int32_t)c.h - 1);
                if (A != 0) {
                    live = (uint32_t)((px1 - px0 + 1) * (py1 - py0 + 1)) <= c.small_area;
                    slow = !live;
                }
            } else {
                const int64_t A64 = (int64_t)(q1.x - q0.x) * (q2.y - q0.y) - (int64_t)(q1.y - q0.y) * (q2.x - q0.x);
                slow = A64 != 0;
            }
        }
    }
    if (live) {
        int32_t x[3] = {q0.x, q1.x, q2.x}, y[3] = {q0.y, q1.y, q2.y};
        float z0 = __int_as_float(q0.z), z1 = __int_as_float(q1.z), z2 = __int_as_float(q2.z);
        if (A < 0) {  // orient to positive area
            x[1] = q2.x, y[1] = q2.y, x[2] = q1.x, y[2] = q1.y;
            z1 = __int_as_float(q2.z), z2 = __int_as_float(q1.z);
        }
        const int32_t Ap = A < 0 ? -A : A;
        const uint32_t bw = (uint32_t)(px1 - px0 + 1), bh = (uint32_t)(py1 - py0 + 1);
        uint32_t bias = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t dx = x[(k + 1) % 3] - x[k], dy = y[(k + 1) % 3] - y[k];
            if (!(dy < 0 || (dy == 0 && dx > 0))) bias |= 1u << k;
        }
        const float dx1 = __int2float_rn(x[1] - x[0]), dy1 = __int2float_rn(y[1] - y[0]);
        const float dx2 = __int2float_rn(x[2] - x[0]), dy2 = __int2float_rn(y[2] - y[0]);
        const float af = __int2float_rn(Ap);
        const float dz1 = fsub(z1, z0), dz2 = fsub(z2, z0);
        const float ra = __frcp_rn(af);
        const float pa = fmul(fsub(fmul(dz1, dy2), fmul(dz2, dy1)), ra);
        const float pb = fmul(fsub(fmul(dz2, dx1), fmul(dz1, dx2)), ra);
        const uint32_t id = (d << 7) | ct;
        if (bw * bh <= kLaneArea) {
            const unsigned long long lo = (unsigned long long)id + 1ull;
            for (uint32_t ly = 0; ly < bh; ++ly)
                for (uint32_t lx = 0; lx < bw; ++lx)
                    small_sample(x, y, bias, z0, pa, pb, px0 + (int32_t)lx, py0 + (int32_t)ly, lo, c);
        } else {
            TriRec& r = recs[lane];
            r.x[0] = x[0], r.x[1] = x[1], r.x[2] = x[2];
            r.y[0] = y[0], r.y[1] = y[1], r.y[2] = y[2];
            r.z0 = z0;
            r.pa = pa;
            r.pb = pb;
            r.inv_bw = 1.0f / (float)bw;
            r.id = id;
            r.bx0 = (uint16_t)px0;
            r.by0 = (uint16_t)py0;
            r.bw = (uint8_t)bw;
            r.bh = (uint8_t)bh;
            r.bias = (uint8_t)bias;
            coop_area = bw * bh;
        }
    }
    // Triangles whose bbox exceeds kQueueArea pixels go to the
    // binned-rectangle queue (one rectangle each), drained by k_raster_big
    // with a warp per rectangle: a meshlet of larger triangles then no
    // longer holds one warp for all of its pixels.  The rest, and anything
    // the full queue refuses, take the warp-cooperative raster below.
    const unsigned mm = __ballot_sync(0xffffffffu, coop_area > kQueueArea);
    if (mm) {
        const int leader = __ffs(mm) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(c.big_count, (uint32_t)__popc(mm));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (coop_area > kQueueArea) {
            const uint32_t slot = base + (uint32_t)__popc(mm & ((1u << lane) - 1u));
            if (slot < c.big_cap) {
                const TriRec& r = recs[lane];
                BigTri t;
                t.x[0] = r.x[0], t.x[1] = r.x[1], t.x[2] = r.x[2];
                t.y[0] = r.y[0], t.y[1] = r.y[1], t.y[2] = r.y[2];
                t.z0 = r.z0, t.pa = r.pa, t.pb = r.pb;
                t.id = r.id;
                t.px0 = r.bx0, t.py0 = r.by0;
                t.px1 = (uint16_t)(r.bx0 + r.bw - 1), t.py1 = (uint16_t)(r.by0 + r.bh - 1);
                t.view = c.view;
                t._pad = 0;
                c.big[slot] = t;
                coop_area = 0;
            } else {
                report(c.status, kStatusQueueOverflow, slot);
            }
        }
    }
    if (__ballot_sync(0xffffffffu, coop_area != 0) == 0) return slow;
    // Warp-cooperative raster: an inclusive scan of the bbox areas spreads
    // the pixels of the larger small triangles evenly over the lanes.
    uint32_t incl = coop_area;
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
        small_sample(r.x, r.y, r.bias, r.z0, r.pa, r.pb, (int32_t)(r.bx0 + lx), (int32_t)(r.by0 + ly),
                     (unsigned long long)r.id + 1ull, c);
    }
    __syncwarp();
    return slow;
}

// Warp-per-meshlet raster.  The fast instance (SLOW = false) handles every
// triangle that needs no clipping and fits the cooperative small-triangle
// path, and appends a meshlet that has any other triangle to the view's
// deferred list.  The slow instance (SLOW = true) re-runs those meshlets and
// handles only the remaining triangles (homogeneous clipping, large or
// off-screen-spanning triangles), so the fast instance calls no function.
template <int WARPS, bool SLOW>
__global__ void __launch_bounds__(WARPS * 32, (SLOW ? 16 : VKGV_RASTER_WARPS_PER_SM) / WARPS) k_raster(RasterParams P) {
    pdl_begin();
    __shared__ float4 s_clip[WARPS][64];
    // per vertex: {X, Y (28.8), Z bits, flags} read with one 16-byte load
    __shared__ int4 s_vtx[WARPS][64];
    // the meshlet's triangle-index bytes (<= 126 triangles)
    __shared__ uint32_t s_idx[WARPS][96];
    __shared__ TriRec s_tri[WARPS][32];
    // ring of compacted candidate triangle indices (fast instance)
    __shared__ uint8_t s_ring[WARPS][64];
    __shared__ uint32_t s_end[WARPS][32];
    __shared__ float s_mvp[WARPS][16];
    __shared__ float s_tdet[WARPS];
    __shared__ float s_vp[WARPS][16];
    // exclusive prefix of the views' work counts: view v owns the global
    // work items [s_pre[v], s_pre[v + 1])
    __shared__ uint32_t s_pre[kRasterMaxViews + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nv = P.nviews;
    for (uint32_t v = threadIdx.x; v < nv; v += blockDim.x) {
        const uint32_t* l;
        uint32_t n, f;
        view_work<SLOW>(P, P.views[v], l, n, f);
        s_pre[v + 1] = n;
    }
    if (threadIdx.x == 0) s_pre[0] = 0;
    __syncthreads();
    if (warp == 0) {
        // inclusive scan of s_pre[1..nv]: lane-contiguous segments, then a
        // warp scan of the segment sums
        const uint32_t seg = (nv + 31) / 32, b = 1 + lane * seg, e = min(b + seg, nv + 1);
        uint32_t sum = 0;
        for (uint32_t i = b; i < e; ++i) sum += s_pre[i];
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        uint32_t run = incl - sum;
        for (uint32_t i = b; i < e; ++i) {
            run += s_pre[i];
            s_pre[i] = run;
        }
    }
    __syncthreads();
    const uint32_t total = s_pre[nv];
    const uint32_t slot = P.lists.deferred_slot;
    const uint32_t defer_cap = P.S.draw_count;
    float4* clip = s_clip[warp];
    int4* svtx = s_vtx[warp];
    uint32_t* sidx = s_idx[warp];
    const uint8_t* sidx8 = reinterpret_cast<const uint8_t*>(sidx);
    TriRec* recs = s_tri[warp];
    uint32_t* ends = s_end[warp];
    // Warps take runs of `grab` consecutive work items from one counter, so
    // views are drawn roughly in order (their depth buffers stay in L2) and
    // no warp idles while work is left.
    const uint32_t warps_total = gridDim.x * WARPS;
    const uint32_t grab = max(1u, min(32u, total / (warps_total * 8u)));
    uint32_t cur_v = 0xffffffffu, cur_t = 0xffffffffu;  // view and node of s_vp / s_mvp
    const DeviceView* Vp = P.views;
    // the warp's raster context lives in shared memory (fewer live registers)
    __shared__ RasterCtx s_ctx[WARPS];
    RasterCtx& c = s_ctx[warp];
    if (lane == 0) {
        c.big = P.big;
        c.big_count = P.big_count;
        c.big_cap = P.big_cap;
        c.small_area = P.small_area;
        c.chunk = P.chunk;
        c.status = P.status;
    }
    // Per-meshlet headers of the current run, resolved one item per lane so
    // that the dependent loads (list entry -> draw -> primitive -> meshlet
    // record, material) of up to 32 meshlets are in flight together instead
    // of one meshlet after another.
    __shared__ ItemHeader s_hdr[WARPS][32];
    ItemHeader* hdr = s_hdr[warp];
    // the next run is requested while the current one is drawn, so the
    // atomic's round trip is off the critical path
    // Warps beyond the first `total` have nothing to take (each of the
    // first `total` grabs returns a distinct item), so they skip the counter.
    uint32_t next = 0xffffffffu;
    if (lane == 0 && blockIdx.x * WARPS + warp < total) next = atomicAdd(P.work, grab);
    for (;;) {
        const uint32_t base = __shfl_sync(0xffffffffu, next, 0);
        if (base >= total) break;
        if (lane == 0) next = atomicAdd(P.work, grab);
        const uint32_t stop = min(base + grab, total);
        {
            const uint32_t g = base + (uint32_t)lane;
            ItemHeader h;
            h.d = 0xffffffffu;
            h.v = 0;
            h.bad = 1;
            if (g < stop) {
                // the view holding g: the last v with s_pre[v] <= g
                uint32_t v = 0, hi = nv;
                while (v + 1 < hi) {
                    const uint32_t mid = (v + hi) >> 1;
                    if (s_pre[mid] <= g) v = mid;
                    else hi = mid;
                }
                const uint32_t* list;
                uint32_t n, first;
                view_work<SLOW>(P, P.views[v], list, n, first);
                const uint32_t d = list[first + (g - s_pre[v])];
                h.v = v;
                h.d = d;
                if (d < P.S.draw_count) {
                    const vkgv_meshlet_draw dr = P.S.draws[d];
                    const vkgv_primitive* prim = &P.S.prims[dr.primitive_index];
                    if (dr.meshlet_index < prim->meshlet_count) {
                        const vkgv_meshlet* ml =
                            reinterpret_cast<const vkgv_meshlet*>(prim->meshlet_buffer) + dr.meshlet_index;
                        const uint32_t vc = ml->vertex_count, tc = ml->triangle_count;
                        if (vc <= VKGV_MAX_VERTICES && tc <= VKGV_MAX_PRIMITIVES) {
                            h.vidx = reinterpret_cast<const uint32_t*>(prim->vertex_index_buffer) + ml->vertex_offset;
                            h.tri = reinterpret_cast<const uint8_t*>(prim->primitive_index_buffer) + ml->triangle_offset;
                            h.verts = reinterpret_cast<const vkgv_vertex*>(prim->vertex_buffer);
                            h.transform = dr.transform_index;
                            h.vc = (uint8_t)vc;
                            h.tc = (uint8_t)tc;
                            h.double_sided = P.S.mats[prim->material_index].double_sided != 0 ? 1 : 0;
                            h.bad = 0;
                        }
                    }
                }
            }
            __syncwarp();  // every lane is done with the previous run's headers
            hdr[lane] = h;
        }
        __syncwarp();
        for (uint32_t k = 0; k < stop - base; ++k) {
            const ItemHeader& H = hdr[k];
            const uint32_t v = H.v, d = H.d;
            if (H.bad) {
                if (lane == 0) report(P.status, kStatusBadIndex, d);
                continue;
            }
            if (v != cur_v) {
                cur_v = v;
                cur_t = 0xffffffffu;
                Vp = P.views + v;
                __syncwarp();
                if (lane == 0) {
                    c.depth = Vp->depth_id;
                    c.w = Vp->w;
                    c.h = Vp->h;
                    c.hw = 0.5f * (float)Vp->w;
                    c.hh = 0.5f * (float)Vp->h;
                    c.view = P.view_base + v;
                }
                if (lane < 16) s_vp[warp][lane] = Vp->cam->view_projection[lane];
                __syncwarp();
            }
            const DeviceView& V = *Vp;
            const uint32_t vc = H.vc, tc = H.tc;
            const uint32_t* vidx = H.vidx;
            const uint8_t* tri = H.tri;
            const vkgv_vertex* verts = H.verts;
            const bool double_sided = H.double_sided != 0;
            const uint32_t transform_index = H.transform;
            // mvp = VP * M, one element per lane (lanes 0-15); lane 16 takes the
            // sign source determinant(M) of visbuffer.mesh.glsl:71.
            // Consecutive items of a run mostly come from one node (the draw
            // list is node-major): its matrix and sign are then already here.
            const float* Mg = P.S.transforms + 16 * (size_t)transform_index;
            const bool have_tdet = P.S.tdets != nullptr && transform_index < P.S.transform_count;
            const bool same_node = transform_index == cur_t;
            cur_t = transform_index;
            if (same_node) {
            } else if (lane < 16 && V.mvps && transform_index < P.S.transform_count) {
                s_mvp[warp][lane] = __ldg(V.mvps + 16 * (size_t)transform_index + lane);
            } else if (lane < 16) {
                const int cc = lane >> 2, j = lane & 3;
                const float4 mc = __ldg(reinterpret_cast<const float4*>(Mg) + cc);
                s_mvp[warp][lane] = fadd(fadd(fadd(fmul(s_vp[warp][0 * 4 + j], mc.x), fmul(s_vp[warp][1 * 4 + j], mc.y)),
                                              fmul(s_vp[warp][2 * 4 + j], mc.z)),
                                         fmul(s_vp[warp][3 * 4 + j], mc.w));
            } else if (lane == 16 && have_tdet) {
                s_tdet[warp] = P.S.tdets[transform_index];
            } else if (lane == 16) {
                float M[16];
    #pragma unroll
                for (int q = 0; q < 16; ++q) M[q] = __ldg(Mg + q);
                s_tdet[warp] = det4(M);
            }
            if (!same_node) __syncwarp();
            const float tdet = s_tdet[warp];
            const float* mvp = s_mvp[warp];
            // Vertex stage: clip position, outcode, guard flag and the 28.8 snap,
            // each computed once per meshlet vertex (two per lane).  All global
            // loads of the stage, and the triangle-index words (32-bit loads
            // when the block is 4-byte aligned, as meshoptimizer pads each
            // block to 4), are issued before any of the math.
            const uint32_t nbytes = 3 * tc, nwords = (nbytes + 3) / 4;  // <= 95 words
            const bool tri_words = (reinterpret_cast<uintptr_t>(tri) & 3u) == 0;
            uint32_t tw[3] = {0u, 0u, 0u};
            if (tri_words) {
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    if (lane + 32u * q < nwords) tw[q] = __ldg(reinterpret_cast<const uint32_t*>(tri) + lane + 32 * q);
            }
            const bool h0 = (uint32_t)lane < vc, h1 = (uint32_t)lane + 32u < vc;
            const vkgv_vertex* vx0 = verts + (h0 ? __ldg(vidx + lane) : 0u);
            const vkgv_vertex* vx1 = verts + (h1 ? __ldg(vidx + lane + 32) : 0u);
            float2 xy0 = make_float2(0.0f, 0.0f), xy1 = xy0;
            float zz0 = 0.0f, zz1 = 0.0f;
            if (h0) {
                xy0 = __ldg(reinterpret_cast<const float2*>(vx0->position));
                zz0 = __ldg(&vx0->position[2]);
            }
            if (h1) {
                xy1 = __ldg(reinterpret_cast<const float2*>(vx1->position));
                zz1 = __ldg(&vx1->position[2]);
            }
            auto vertex = [&](uint32_t k, float px, float py, float pz) {
                float r[4];
                m4v(mvp, px, py, pz, 1.0f, r);
                const float4 cv = make_float4(r[0], r[1], r[2], r[3]);
                clip[k] = cv;
                int32_t X = 0, Y = 0;
                float Z = 0.0f;
                uint32_t fl = (uint32_t)outcode(cv);
                if (outside_guard(cv)) fl |= kFlagGuard;
                if (snap(cv, c, X, Y, Z)) fl |= kFlagSnapped;
                svtx[k] = make_int4(X, Y, __float_as_int(Z), (int)fl);
            };
            if (h0) vertex(lane, xy0.x, xy0.y, zz0);
            if (h1) vertex(lane + 32, xy1.x, xy1.y, zz1);
            if (tri_words) {
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    if (lane + 32u * q < nwords) sidx[lane + 32 * q] = tw[q];
            } else {
                uint8_t* b = reinterpret_cast<uint8_t*>(sidx);
                for (uint32_t k = lane; k < nbytes; k += 32) b[k] = __ldg(tri + k);
            }
            __syncwarp();
            bool any_slow = false;
            if constexpr (SLOW) {
                // Deferred meshlet: only the triangles the fast instance
                // skipped, 32 per round; the round's binned triangles are
                // queued together when the warp has reconverged.
                JobList jobs;
                jobs.count = 0;
                for (uint32_t tb = 0; tb < tc; tb += 32) {
                    const uint32_t t = tb + (uint32_t)lane;
                    if (t < tc) {
                        TriClass k;
                        const uint32_t i0 = sidx8[3 * t], i1 = sidx8[3 * t + 1], i2 = sidx8[3 * t + 2];
                        const int kind = classify<true>(i0, i1, i2, vc, svtx, clip, double_sided, tdet, c, d, k);
                        if (kind == kSlowClip) {
                            raster_clipped(clip[i0], clip[i1], clip[i2],
                                           (((uint32_t)k.q0.w | (uint32_t)k.q1.w | (uint32_t)k.q2.w) & (OC_ZLO | OC_ZHI)) != 0,
                                           (d << 7) | t, c, jobs);
                        } else if (kind == kSlowSetup) {
                            setup_and_raster(k.q0.x, k.q0.y, __int_as_float(k.q0.z), k.q1.x, k.q1.y,
                                             __int_as_float(k.q1.z), k.q2.x, k.q2.y, __int_as_float(k.q2.z),
                                             (d << 7) | t, c, jobs);
                        }
                    }
                    __syncwarp();
                    flush_jobs(jobs, c, lane);
                }
            } else {
                // Pre-filter 32 triangles per round (outcodes, snap, a pixel
                // centre in the bbox); the candidates are compacted into a
                // ring so that the backface, area and size tests, the setup and
                // the raster run on full warps (at most about a quarter of the
                // triangles of a dense meshlet have a sample in their bbox).
                uint8_t* ring = s_ring[warp];
                uint32_t head = 0, pending = 0;
                for (uint32_t tbase = 0; tbase < tc; tbase += 32) {
                    const uint32_t t = tbase + lane;
                    int kind = 0;
                    if (t < tc) kind = prefilter(sidx8[3 * t], sidx8[3 * t + 1], sidx8[3 * t + 2], vc, svtx, c, d);
                    any_slow |= kind == 2;
                    const uint32_t fm = __ballot_sync(0xffffffffu, kind == 1);
                    if (kind == 1) ring[(head + pending + __popc(fm & ((1u << lane) - 1u))) & 63u] = (uint8_t)t;
                    pending += __popc(fm);
                    const bool last = tbase + 32 >= tc;
                    while (pending >= 32 || (last && pending > 0)) {
                        __syncwarp();
                        const uint32_t n = min(pending, 32u);
                        const uint32_t ct = lane < n ? ring[(head + lane) & 63u] : 0xffffffffu;
                        __syncwarp();
                        any_slow |= raster_small(ct, sidx8, svtx, clip, double_sided, tdet, d, c, recs, ends, lane);
                        head = (head + n) & 63u;
                        pending -= n;
                    }
                }
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
    // The last CTA to finish resets the work counters for the next launch.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(P.work + 1, 1u) == gridDim.x - 1) {
            P.work[0] = 0;
            P.work[1] = 0;
        }
    }
}

// Drains the binned rectangles: one warp per rectangle, its pixels spread
// over the lanes in row-major order (eight rectangles in flight per CTA).
__global__ void __launch_bounds__(256) k_raster_big(const BigTri* __restrict__ q, const uint32_t* count,
                                                    uint32_t cap, const DeviceView* __restrict__ views) {
    pdl_begin();
    const uint32_t n = min(*count, cap);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < n; e += warps) {
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
        const uint32_t bw = (uint32_t)t.px1 - t.px0 + 1u, area = bw * ((uint32_t)t.py1 - t.py0 + 1u);
        // floor((i + 0.5) / bw) from the float reciprocal is exact here: the
        // quotient stays at least 0.5 / bw from an integer and i < 4096.
        const float inv_bw = 1.0f / (float)bw;
        for (uint32_t i = lane; i < area; i += 32) {
            const uint32_t ly = (uint32_t)(((float)i + 0.5f) * inv_bw);
            const int px = (int)(t.px0 + (i - ly * bw)), py = (int)(t.py0 + ly);
            const int32_t sx = px * 256 + 128, sy = py * 256 + 128;
            bool covered = true;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int a = k, b = (k + 1) % 3;
                const int64_t ev = (int64_t)(t.x[b] - t.x[a]) * (sy - t.y[a]) -
                                   (int64_t)(t.y[b] - t.y[a]) * (sx - t.x[a]);
                covered = covered && ev >= bias[k];
            }
            if (!covered) continue;
            float z = __fmaf_rn(t.pa, __int2float_rn(sx - t.x[0]), __fmaf_rn(t.pb, __int2float_rn(sy - t.y[0]), t.z0));
            if (!(z > 0.0f)) z = 0.0f;
            if (z > 1.0f) z = 1.0f;
            plot(depth + (size_t)py * w + px, ((unsigned long long)__float_as_uint(z) << 32) | lo);
        }
    }
}

// One wave of CTAs: every warp stays resident and takes work until none is
// left.
template <int WARPS>
void launch_variant(const RasterParams& P, uint32_t sm_count, uint32_t blocks_override, cudaStream_t stream) {
    const uint32_t fast = blocks_override ? blocks_override : sm_count * (VKGV_RASTER_WARPS_PER_SM / WARPS);
    const uint32_t slow = blocks_override ? blocks_override : sm_count * (16 / WARPS > 0 ? 16 / WARPS : 1);
    launch_pdl(k_raster<WARPS, false>, dim3(fast), dim3(WARPS * 32), 0, stream, P);
    launch_pdl(k_raster<WARPS, true>, dim3(slow), dim3(WARPS * 32), 0, stream, P);
}

}  // namespace

void launch_raster(const SceneArgs& S, const DeviceView* views, uint32_t nviews, const RasterLists& lists,
                   const RasterConfig& cfg, BigTri* big, uint32_t* big_count, uint32_t big_capacity,
                   uint32_t* work, uint32_t* status, uint32_t sm_count, cudaStream_t stream, cudaEvent_t between) {
    RasterParams P;
    P.S = S;
    P.lists = lists;
    P.big = big;
    P.big_count = big_count;
    P.big_cap = big_capacity;
    P.small_area = cfg.small_area;
    P.chunk = cfg.chunk;
    P.status = status;
    P.work = work;
    for (uint32_t v0 = 0; v0 < nviews; v0 += kRasterMaxViews) {
        P.views = views + v0;
        P.nviews = nviews - v0 < kRasterMaxViews ? nviews - v0 : kRasterMaxViews;
        P.view_base = v0;
        switch (cfg.warps_per_cta) {
            case 1: launch_variant<1>(P, sm_count, cfg.blocks_per_view, stream); break;
            case 2: launch_variant<2>(P, sm_count, cfg.blocks_per_view, stream); break;
            case 8: launch_variant<8>(P, sm_count, cfg.blocks_per_view, stream); break;
            default: launch_variant<4>(P, sm_count, cfg.blocks_per_view, stream); break;
        }
    }
    if (between) cudaEventRecord(between, stream);
    // Exactly one wave of drain CTAs: its warps stride over the queue
    // statically, so a partial second wave (8 CTAs per SM against 5
    // resident) finished late: single view 36.9 -> 34.8 us, 256 views
    // 0.125 -> 0.111 ms.  (Warps taking rectangles from a counter instead
    // were 1.3-2.9x slower: same-address atomics.)
    static std::atomic<int> resident[64];
    int dev = 0;
    cudaGetDevice(&dev);
    int per_sm = dev >= 0 && dev < 64 ? resident[dev].load(std::memory_order_relaxed) : 0;
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster_big, 256, 0) != cudaSuccess || per_sm <= 0)
            per_sm = 4;
        if (dev >= 0 && dev < 64) resident[dev].store(per_sm, std::memory_order_relaxed);
    }
    launch_pdl(k_raster_big, dim3(sm_count * (uint32_t)per_sm), dim3(256), 0, stream, (const BigTri*)big,
               (const uint32_t*)big_count, big_capacity, views);
}

}  // namespace vkgv
