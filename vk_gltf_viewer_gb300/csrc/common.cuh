// Shared device-side definitions for the vkgv kernels (sm_103a).
//
// Every floating-point operation that feeds a compared result (survivor set,
// visibility IDs, HiZ mips) is written with explicit round-to-nearest
// intrinsics so that the compiler cannot contract or reorder it; the order
// of operations is the pinned one that the CPU oracle also uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vkgv.h"

static_assert(sizeof(vkgv_meshlet) == 36, "glsl::Meshlet is 36 bytes");
static_assert(sizeof(vkgv_vertex) == 24, "glsl::Vertex is 24 bytes");
static_assert(sizeof(vkgv_meshlet_draw) == 12, "glsl::MeshletDraw is 12 bytes");
static_assert(sizeof(vkgv_primitive) == 64, "glsl::Primitive is 64 bytes");
static_assert(alignof(vkgv_primitive) == 8, "glsl::Primitive is 8-aligned");
static_assert(sizeof(vkgv_material) == 48, "glsl::Material is 48 bytes");
static_assert(sizeof(vkgv_camera) == 352, "glsl::Camera is 352 bytes");

namespace vkgv {

// Device status word codes (first violation wins).
enum StatusCode : uint32_t {
    kStatusOk = 0,
    kStatusBadIndex = 1,        // draw/primitive/meshlet/vertex index out of range
    kStatusQueueOverflow = 2,   // binned-triangle queue full (handled inline, reported)
    kStatusListOverflow = 3,    // survivor list capacity exceeded
    kStatusTimeout = 4,         // a bounded wait ran out
};

// Per-view state as the kernels see it (built by the host from vkgv_view).
struct DeviceView {
    const vkgv_camera* cam;
    uint32_t w, h;
    const float* prev_pyr;
    uint32_t prev_w0, prev_h0, prev_levels;
    uint32_t pyr_levels;
    float* pyr;
    unsigned long long* depth_id;
    uint32_t* ids;
    uint32_t* rgba;
    uint32_t* survivors;        // pass-1 survivors at [0, c[0]), pass-2 at [c[0], c[0]+c[2])
    uint32_t* survivor_count;   // user-visible total (written by the finalize step)
    uint32_t* rejected;         // pass-1 occlusion rejects (scratch)
    uint32_t* deferred;         // meshlets with clipped or large triangles (scratch, capacity = draws)
    // scratch counters: [0] pass-1 survivors, [1] rejects, [2] pass-2 survivors,
    // [3] HiZ tiles done, [4..6] deferred meshlets of raster pass 1 / 2 / explicit list
    uint32_t* counters;
    uint32_t survivor_capacity;
    uint32_t _pad;
    float* diff_rgb;            // adjoint: shaded linear RGB output (forward)
    const float* diff_target;   // adjoint: MSE target image (backward)
    const float* diff_grad;     // adjoint: dL/drgb (backward, without a target)
    // view_projection * M per node (16 floats each, computed by the clear), or null
    const float* mvps;
    // prev_view_projection * M per node (motion-vector frames only), or null
    const float* prev_mvps;
    uint32_t* motion;           // two binary16 per pixel (x low), or null
    // per node: the raster eye in the node's object space and 1 (0 for a
    // singular transform or no eye), for the cone test; filled by the clear
    const float4* eyes;
    // per pass-1 occlusion reject (same slot as `rejected`): the HiZ sample
    // that rejected it (nearest AABB depth, level, texel footprint), so that
    // pass 2 can repeat the lookup on the new pyramid without projecting the
    // box again when the occlusion camera and pyramid shape are unchanged;
    // null: pass 2 recomputes
    unsigned long long* reject_samples;
};

struct SceneArgs {
    const vkgv_meshlet_draw* draws;
    const float* transforms;
    const vkgv_primitive* prims;
    const vkgv_material* mats;
    const vkgv_texture* textures;
    uint32_t draw_count;
    uint32_t texture_count;
    const uint64_t* cone_table;   // per primitive: device address of its cones, or 0
    uint32_t primitive_count;
    uint32_t transform_count;
    const float* tdets;           // determinant(M) per node (computed by the clear), or null
};

// One binned (large) triangle chunk: a sub-rectangle of a snapped triangle.
struct BigTri {
    int32_t x[3], y[3];       // 28.8 fixed point, positive orientation
    float z0, pa, pb;         // depth plane
    uint32_t id;              // visbuffer id
    uint16_t px0, py0, px1, py1;  // inclusive pixel rectangle
    uint32_t view;
    uint32_t _pad;
};
static_assert(sizeof(BigTri) == 56, "BigTri layout");

// ------------------------------------------------------------ pinned math
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// GLSL 4.60 min/max/clamp definitions.
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

// r_j = ((m0j*v0 + m1j*v1) + m2j*v2) + m3j*v3, column-major m[c*4 + j].
__device__ __forceinline__ void m4v(const float* m, float v0, float v1, float v2, float v3, float r[4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
        r[j] = fadd(fadd(fadd(fmul(m[0 * 4 + j], v0), fmul(m[1 * 4 + j], v1)), fmul(m[2 * 4 + j], v2)),
                    fmul(m[3 * 4 + j], v3));
}

// r = a * b (column-major).
__device__ __forceinline__ void m4m(const float* a, const float* b, float* r) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            r[c * 4 + j] = fadd(fadd(fadd(fmul(a[0 * 4 + j], b[c * 4 + 0]), fmul(a[1 * 4 + j], b[c * 4 + 1])),
                                     fmul(a[2 * 4 + j], b[c * 4 + 2])),
                                fmul(a[3 * 4 + j], b[c * 4 + 3]));
}

// determinant(mat3(P, Q, R)) with columns P, Q, R.
__device__ __forceinline__ float det3(float p0, float p1, float p2, float q0, float q1, float q2, float r0,
                                      float r1, float r2) {
    float t1 = fmul(p0, fsub(fmul(q1, r2), fmul(r1, q2)));
    float t2 = fmul(q0, fsub(fmul(p1, r2), fmul(r1, p2)));
    float t3 = fmul(r0, fsub(fmul(p1, q2), fmul(q1, p2)));
    return fadd(fsub(t1, t2), t3);
}

// determinant(mat4) by expansion along column 0.
__device__ __forceinline__ float det4(const float* m) {
    float d[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float c1[3], c2[3], c3[3];
        int k = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j == r) continue;
            c1[k] = m[1 * 4 + j];
            c2[k] = m[2 * 4 + j];
            c3[k] = m[3 * 4 + j];
            ++k;
        }
        d[r] = det3(c1[0], c1[1], c1[2], c2[0], c2[1], c2[2], c3[0], c3[1], c3[2]);
    }
    return fsub(fadd(fsub(fmul(m[0], d[0]), fmul(m[1], d[1])), fmul(m[2], d[2])), fmul(m[3], d[3]));
}

// Eye position of a view-projection (the point where clip x, y and w are 0),
// by Cramer's rule on rows 0, 1 and 3.  Returns false when singular.
__device__ __forceinline__ bool eye_from_vp(const float* vp, float e[3]) {
    const float a0x = vp[0], a0y = vp[4], a0z = vp[8], b0 = -vp[12];
    const float a1x = vp[1], a1y = vp[5], a1z = vp[9], b1 = -vp[13];
    const float a2x = vp[3], a2y = vp[7], a2z = vp[11], b2 = -vp[15];
    const float det = det3(a0x, a0y, a0z, a1x, a1y, a1z, a2x, a2y, a2z);
    if (!(det != 0.0f)) return false;
    e[0] = fdiv(det3(b0, a0y, a0z, b1, a1y, a1z, b2, a2y, a2z), det);
    e[1] = fdiv(det3(a0x, b0, a0z, a1x, b1, a1z, a2x, b2, a2z), det);
    e[2] = fdiv(det3(a0x, a0y, b0, a1x, a1y, b1, a2x, a2y, b2), det);
    return true;
}

// Conservative meshlet backface test in object space: every triangle of
// the meshlet faces away from the eye by a margin of 1e-3 (L + r) when
//   d*c + sqrt(L^2 - d^2)*s < -(r + 1e-3 (L + r)),
// with L = |eye - center|, d = axis . (eye - center), c the cone cutoff and
// s = sqrt(1 - c^2).  `M` is the instance transform (column-major).
// The eye in the object space of instance transform M (Cramer's rule on
// the upper 3x3); false when that is singular.  It depends on the node and
// the view only, so whole frames take it from a per-view node table.
__device__ __forceinline__ bool object_eye(const float* M, const float* eye, float o[3]) {
    const float det = det3(M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]);
    if (!(det != 0.0f)) return false;
    const float vx = fsub(eye[0], M[12]), vy = fsub(eye[1], M[13]), vz = fsub(eye[2], M[14]);
    o[0] = fdiv(det3(vx, vy, vz, M[4], M[5], M[6], M[8], M[9], M[10]), det);
    o[1] = fdiv(det3(M[0], M[1], M[2], vx, vy, vz, M[8], M[9], M[10]), det);
    o[2] = fdiv(det3(M[0], M[1], M[2], M[4], M[5], M[6], vx, vy, vz), det);
    return true;
}

// The test itself for an object-space eye (ox, oy, oz).
__device__ __forceinline__ bool cone_culled_at(const vkgv_meshlet_cone& cone, float ox, float oy, float oz) {
    const float c = cone.cutoff;
    if (!(c > 0.0f)) return false;
    const float wx = fsub(ox, cone.center[0]), wy = fsub(oy, cone.center[1]), wz = fsub(oz, cone.center[2]);
    const float L2 = fadd(fadd(fmul(wx, wx), fmul(wy, wy)), fmul(wz, wz));
    const float d = fadd(fadd(fmul(cone.axis[0], wx), fmul(cone.axis[1], wy)), fmul(cone.axis[2], wz));
    const float s = __fsqrt_rn(fmaxf(fsub(1.0f, fmul(c, c)), 0.0f));
    const float perp = __fsqrt_rn(fmaxf(fsub(L2, fmul(d, d)), 0.0f));
    const float lhs = fadd(fmul(d, c), fmul(perp, s));
    const float margin = fadd(cone.radius, fmul(1e-3f, fadd(__fsqrt_rn(L2), cone.radius)));
    return lhs < -margin;
}

__device__ __forceinline__ bool cone_culled(const vkgv_meshlet_cone& cone, const float* M, const float* eye) {
    if (!(cone.cutoff > 0.0f)) return false;
    float o[3];
    if (!object_eye(M, eye, o)) return false;
    return cone_culled_at(cone, o[0], o[1], o[2]);
}

__host__ __device__ __forceinline__ uint32_t mip_dim(uint32_t base, uint32_t k) {
    uint32_t v = base >> k;
    return v ? v : 1u;
}

__host__ __device__ __forceinline__ uint64_t mip_offset(uint32_t w0, uint32_t h0, uint32_t level) {
    uint64_t off = 0;
    for (uint32_t k = 0; k < level; ++k) off += (uint64_t)mip_dim(w0, k) * mip_dim(h0, k);
    return off;
}

// HiZ tiling (single-pass reduce): a CTA owns an 8x8 tile of the highest
// tiled level (at most level 4) and the matching 2^k-times larger tiles of
// the levels below it.  Levels with a zero dimension are never tiled.
constexpr int kHizTileLevels = 4;
constexpr int kHizTopTile = 4;

__host__ __device__ __forceinline__ int hiz_tile_levels(uint32_t w, uint32_t h, uint32_t levels) {
    int k = (int)(levels < (uint32_t)kHizTileLevels ? levels : (uint32_t)kHizTileLevels);
    while (k > 0 && ((w >> k) == 0 || (h >> k) == 0)) --k;
    return k;
}

__host__ __device__ __forceinline__ int hiz_tile_edge(int level, int top) { return kHizTopTile << (top - level); }

__host__ __device__ __forceinline__ void hiz_tiles(uint32_t w, uint32_t h, uint32_t levels, uint32_t* tx,
                                                   uint32_t* ty) {
    const int top = hiz_tile_levels(w, h, levels);
    uint32_t nx = 1, ny = 1;
    for (int j = 1; j <= top; ++j) {
        const uint32_t t = (uint32_t)hiz_tile_edge(j, top);
        const uint32_t ax = ((w >> j) + t - 1) / t, ay = ((h >> j) + t - 1) / t;
        nx = ax > nx ? ax : nx;
        ny = ay > ny ? ay : ny;
    }
    *tx = nx;
    *ty = ny;
}

// Texels of one axis of the MIN-reduction LINEAR footprint (pinned rule):
// t = u*size - 0.5; i = floor(t); a = t - i; texel i counts when 1-a != 0,
// texel i+1 when a != 0; clamp-to-edge.  Returns the count (1 or 2).
__device__ __forceinline__ int footprint_axis(float u, uint32_t size, int& i0, int& i1) {
    float t = fsub(fmul(u, (float)size), 0.5f);
    if (!(t >= -1.0f)) t = -1.0f;
    if (!(t <= (float)size)) t = (float)size;
    float fl = floorf(t);
    int i = (int)fl;
    float a = fsub(t, fl);
    int hi = (int)size - 1;
    int n = 0;
    int c0 = i < 0 ? 0 : (i > hi ? hi : i);
    int c1 = i + 1 < 0 ? 0 : (i + 1 > hi ? hi : i + 1);
    if (fsub(1.0f, a) != 0.0f) {
        i0 = c0;
        n = 1;
        if (a != 0.0f) {
            i1 = c1;
            n = 2;
        }
    } else {
        i0 = c1;
        n = 1;
    }
    return n;
}

// Programmatic dependent launch.  A frame's kernels are launched with the
// programmatic-stream-serialisation attribute: each one first lets its
// successor's CTAs be scheduled (they become resident as this grid drains)
// and then waits for its predecessor grid to complete and flush, before it
// reads anything.  Without the attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Device status word: records the first violation (code, detail).
__device__ __forceinline__ void report(uint32_t* status, uint32_t code, uint32_t detail) {
    if (status && atomicCAS(status, 0u, code) == 0u) status[1] = detail;
}

__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }

}  // namespace vkgv
