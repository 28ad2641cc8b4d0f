/*
 * oracle.c — CPU restatement of vk_gltf_viewer's meshlet visibility-buffer
 * path.  TEST INFRASTRUCTURE ONLY (see oracle.h): used by the tests, the
 * smoke check and the benchmark's CPU-baseline leg as the checker; never
 * linked into or called by the product library.
 *
 * Parity status: pinned by hand-derived known-answer cases only (the
 * reference renderer needs a Vulkan mesh-shader device, which does not exist
 * here); parity with the reference's own execution is unpinned beyond them.
 *
 * Build: gcc -O2 -ffp-contract=off -fno-fast-math (no FMA contraction, IEEE
 * division, explicit fmaf only where the pinned rules below name it).
 *
 * Pinned arithmetic (identical in the CUDA kernels):
 *   - mat4 * vec4 / mat4 * mat4: column-major, sums left to right,
 *     ((a0*b0 + a1*b1) + a2*b2) + a3*b3, every operation rounded (no FMA).
 *   - dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z.
 *   - GLSL min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x,
 *     clamp(x,lo,hi) = min(max(x,lo),hi) (GLSL 4.60 built-in definitions).
 *   - determinant(mat3(P,Q,R)) = (P0*(Q1*R2 - R1*Q2) - Q0*(P1*R2 - R1*P2))
 *                                 + R0*(P1*Q2 - Q1*P2).
 *   - floor(log2(m)) of the occlusion test is the exact binary exponent of m;
 *     m <= 0 or NaN gives level 0, +inf the last level.
 *   - Min-reduction sampler (VK_SAMPLER_REDUCTION_MODE_MIN, LINEAR,
 *     CLAMP_TO_EDGE): t = u*size - 0.5 (fp32), i = floor(t), a = t - i;
 *     texel i counts when (1 - a) != 0, texel i+1 when a != 0; result is the
 *     minimum over the counted texels of the 2-D product footprint.
 *   - Raster (Vulkan fixed function, application.cpp:326-340, 830-841):
 *     outcode reject; homogeneous clipping against z >= 0 and z <= w, and
 *     against |x|,|y| <= 256 w (guard band) only when a vertex lies outside
 *     them; viewport x_f = (x/w)*(W/2) + W/2; 8 sub-pixel bits with
 *     round-half-even snapping; pixel centres at +0.5; top-left fill rule;
 *     depth z(S) = fmaf(a, Sx-X0, fmaf(b, Sy-Y0, z0)) from a plane set up in
 *     fp32, clamped to [0, 1]; the GREATER_OR_EQUAL depth test with later
 *     API order winning ties is max over (depth, id).
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* --------------------------------------------------------------- threads */

static int g_threads = 1;

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : (n > 256 ? 256 : n); }
int orc_get_threads(void) { return g_threads; }

typedef void (*orc_range_fn)(void* ctx, int64_t begin, int64_t end, int worker);

typedef struct {
    orc_range_fn fn;
    void* ctx;
    int64_t begin, end;
    int worker;
} orc_job;

static void* orc_job_main(void* p) {
    orc_job* j = (orc_job*)p;
    if (j->begin < j->end) j->fn(j->ctx, j->begin, j->end, j->worker);
    return NULL;
}

/* Static contiguous split of [0, n) over the worker threads. */
static void orc_parallel_for(int64_t n, orc_range_fn fn, void* ctx) {
    int t = g_threads;
    if (t <= 1 || n < 2) {
        fn(ctx, 0, n, 0);
        return;
    }
    if (t > n) t = (int)n;
    pthread_t th[256];
    orc_job jobs[256];
    int64_t chunk = (n + t - 1) / t;
    for (int i = 0; i < t; ++i) {
        jobs[i].fn = fn;
        jobs[i].ctx = ctx;
        jobs[i].begin = i * chunk < n ? i * chunk : n;
        jobs[i].end = (i + 1) * chunk < n ? (i + 1) * chunk : n;
        jobs[i].worker = i;
    }
    int started[256];
    for (int i = 1; i < t; ++i) started[i] = pthread_create(&th[i], NULL, orc_job_main, &jobs[i]) == 0;
    orc_job_main(&jobs[0]);
    for (int i = 1; i < t; ++i) {
        if (started[i])
            pthread_join(th[i], NULL);
        else
            orc_job_main(&jobs[i]);
    }
}

/* ---------------------------------------------------------- pinned math */

static inline float gmin(float x, float y) { return y < x ? y : x; }
static inline float gmax(float x, float y) { return x < y ? y : x; }
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

static inline uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

/* r = m * v, column-major m[c*4 + r]. */
static void m4v(const float* m, const float v[4], float r[4]) {
    for (int j = 0; j < 4; ++j)
        r[j] = ((m[0 * 4 + j] * v[0] + m[1 * 4 + j] * v[1]) + m[2 * 4 + j] * v[2]) + m[3 * 4 + j] * v[3];
}

/* r = a * b. */
static void m4m(const float* a, const float* b, float* r) {
    for (int c = 0; c < 4; ++c)
        for (int j = 0; j < 4; ++j)
            r[c * 4 + j] = ((a[0 * 4 + j] * b[c * 4 + 0] + a[1 * 4 + j] * b[c * 4 + 1]) +
                            a[2 * 4 + j] * b[c * 4 + 2]) +
                           a[3 * 4 + j] * b[c * 4 + 3];
}

/* determinant(mat3(P, Q, R)) with P, Q, R the columns. */
static float det3(const float P[3], const float Q[3], const float R[3]) {
    float t1 = P[0] * (Q[1] * R[2] - R[1] * Q[2]);
    float t2 = Q[0] * (P[1] * R[2] - R[1] * P[2]);
    float t3 = R[0] * (P[1] * Q[2] - Q[1] * P[2]);
    return (t1 - t2) + t3;
}

/* determinant(mat4) by expansion along column 0 (only its sign is used,
 * visbuffer.mesh.glsl:71, 94). */
static float det4(const float* m) {
    float d[4];
    for (int r = 0; r < 4; ++r) {
        float c1[3], c2[3], c3[3];
        int k = 0;
        for (int j = 0; j < 4; ++j) {
            if (j == r) continue;
            c1[k] = m[1 * 4 + j];
            c2[k] = m[2 * 4 + j];
            c3[k] = m[3 * 4 + j];
            ++k;
        }
        d[r] = det3(c1, c2, c3);
    }
    return ((m[0] * d[0] - m[1] * d[1]) + m[2] * d[2]) - m[3] * d[3];
}

/* ------------------------------------------------------------- pyramid */

uint32_t orc_pyramid_levels(uint32_t w, uint32_t h) {
    uint32_t mx = w > h ? w : h, l = 0;
    while ((2u << l) <= mx) ++l; /* floor(log2(max(W,H))), application.cpp:472-473 */
    return l;
}

static uint32_t mip_dim(uint32_t base, uint32_t k) {
    uint32_t v = base >> k;
    return v ? v : 1u;
}

static uint64_t mip_offset(uint32_t w0, uint32_t h0, uint32_t level) {
    uint64_t off = 0;
    for (uint32_t k = 0; k < level; ++k) off += (uint64_t)mip_dim(w0, k) * mip_dim(h0, k);
    return off;
}

uint64_t orc_pyramid_floats(uint32_t w, uint32_t h) {
    return mip_offset(w >> 1, h >> 1, orc_pyramid_levels(w, h));
}

/* Texels of one axis in the min-reduction footprint (pinned rule above). */
static int footprint_axis(float u, uint32_t size, int out[2]) {
    float t = u * (float)size - 0.5f;
    if (!(t >= -1.0f)) t = -1.0f; /* also maps NaN; clamp-to-edge makes this neutral */
    if (!(t <= (float)size)) t = (float)size;
    float fl = floorf(t);
    int i = (int)fl;
    float a = t - fl;
    int n = 0;
    int hi = (int)size - 1;
    if (1.0f - a != 0.0f) out[n++] = i < 0 ? 0 : (i > hi ? hi : i);
    if (a != 0.0f) out[n++] = i + 1 < 0 ? 0 : (i + 1 > hi ? hi : i + 1);
    return n;
}

/* Min-reduction bilinear sample of a w x h single-level image. */
float orc_min_sample(const float* img, uint32_t w, uint32_t h, float u, float v) {
    int xs[2], ys[2];
    int nx = footprint_axis(u, w, xs), ny = footprint_axis(v, h, ys);
    float r = 0.0f;
    int first = 1;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            float t = img[(size_t)ys[j] * w + xs[i]];
            r = first ? t : gmin(r, t);
            first = 0;
        }
    return r;
}

/* --------------------------------------------------------------- culling */

/* isAabbInFrustum, shaders/culling.h.glsl:8-19. */
int orc_frustum_visible(const float c[3], const float e[3], const float planes[24]) {
    for (int i = 0; i < 6; ++i) {
        const float* p = planes + 4 * i;
        float radius = (e[0] * fabsf(p[0]) + e[1] * fabsf(p[1])) + e[2] * fabsf(p[2]);
        float distance = ((p[0] * c[0] + p[1] * c[1]) + p[2] * c[2]) - p[3];
        if (-radius > distance) return 0;
    }
    return 1;
}

/* Eye of a view-projection: the point with clip x = y = w = 0, by Cramer's
 * rule on rows 0, 1, 3 (pinned like the kernel).  0 when singular. */
static int eye_from_vp(const float* vp, float e[3]) {
    const float a0[3] = {vp[0], vp[4], vp[8]}, a1[3] = {vp[1], vp[5], vp[9]}, a2[3] = {vp[3], vp[7], vp[11]};
    const float b0 = -vp[12], b1 = -vp[13], b2 = -vp[15];
    float det = det3(a0, a1, a2);
    if (!(det != 0.0f)) return 0;
    const float x0[3] = {b0, a0[1], a0[2]}, x1[3] = {b1, a1[1], a1[2]}, x2[3] = {b2, a2[1], a2[2]};
    const float y0[3] = {a0[0], b0, a0[2]}, y1[3] = {a1[0], b1, a1[2]}, y2[3] = {a2[0], b2, a2[2]};
    const float z0[3] = {a0[0], a0[1], b0}, z1[3] = {a1[0], a1[1], b1}, z2[3] = {a2[0], a2[1], b2};
    e[0] = det3(x0, x1, x2) / det;
    e[1] = det3(y0, y1, y2) / det;
    e[2] = det3(z0, z1, z2) / det;
    return 1;
}

/* Conservative meshlet backface test in object space (the cone-culling
 * addition): every triangle faces away from the eye by 1e-3 (L + r) when
 * d*c + sqrt(L^2 - d^2)*s < -(r + 1e-3 (L + r)). */
static int cone_culled(const orc_cone* cone, const float* M, const float* eye) {
    const float c = cone->cutoff;
    if (!(c > 0.0f)) return 0;
    const float C0[3] = {M[0], M[1], M[2]}, C1[3] = {M[4], M[5], M[6]}, C2[3] = {M[8], M[9], M[10]};
    const float det = det3(C0, C1, C2);
    if (!(det != 0.0f)) return 0;
    const float v[3] = {eye[0] - M[12], eye[1] - M[13], eye[2] - M[14]};
    const float ox = det3(v, C1, C2) / det, oy = det3(C0, v, C2) / det, oz = det3(C0, C1, v) / det;
    const float wx = ox - cone->center[0], wy = oy - cone->center[1], wz = oz - cone->center[2];
    const float L2 = (wx * wx + wy * wy) + wz * wz;
    const float d = (cone->axis[0] * wx + cone->axis[1] * wy) + cone->axis[2] * wz;
    const float s = sqrtf(fmaxf(1.0f - c * c, 0.0f));
    const float perp = sqrtf(fmaxf(L2 - d * d, 0.0f));
    const float lhs = d * c + perp * s;
    const float margin = cone->radius + 1e-3f * (sqrtf(L2) + cone->radius);
    return lhs < -margin;
}

/* Exact floor(log2(m)) clamped to [0, levels-1] (pinned rule above). */
static int hiz_level(float m, uint32_t levels) {
    int top = (int)levels - 1;
    if (!(m > 0.0f)) return 0;
    if (isinf(m)) return top;
    int e;
    frexpf(m, &e); /* m = f * 2^e, f in [0.5, 1) */
    int l = e - 1;
    return l < 0 ? 0 : (l > top ? top : l);
}

/* One draw of the task shader (visbuffer.task.glsl:44-65).  Returns 1 if
 * visible; *occluded is set when the frustum test passed and the occlusion
 * test failed. */
static int ctz32(uint32_t v) {
    int n = 0;
    while (!(v & 1u)) {
        v >>= 1;
        ++n;
    }
    return n;
}

/* The fine occlusion addition (ORC_CULL_OCCLUSION_FINE; no counterpart in
 * the reference).  For a draw the HiZ test kept, the pyramid texels under
 * its projected box [mn0, mx0] x [mn1, mx1] (level-0 texel units, widened by
 * 1/64 texel) are read at the finest level, among those reached from the
 * depth buffer by exact halvings (view width and height divisible by
 * 2^(level+1)), where they are at most 4 x 4; the draw is occluded when
 * every one of them is >= mx2, the box's nearest depth (the comparison of
 * visbuffer.task.glsl:64).  Only with all eight corners in front of the
 * camera (w > 0); otherwise, or with no such level, the HiZ verdict stands. */
static int fine_occluded(const orc_pyramid* pyr, uint32_t vw, uint32_t vh, float mn0, float mx0, float mn1,
                         float mx1, float mx2) {
    if ((vw & 1u) || (vh & 1u) || vw == 0 || vh == 0) return 0;
    int top = ctz32(vw) < ctz32(vh) ? ctz32(vw) - 1 : ctz32(vh) - 1;
    if (top > (int)pyr->levels - 1) top = (int)pyr->levels - 1;
    const int pw = (int)pyr->width, ph = (int)pyr->height;
    int i0 = (int)floorf(mn0 * (float)pw - 0.015625f), i1 = (int)floorf(mx0 * (float)pw + 0.015625f);
    int j0 = (int)floorf(mn1 * (float)ph - 0.015625f), j1 = (int)floorf(mx1 * (float)ph + 0.015625f);
    i0 = i0 < 0 ? 0 : (i0 > pw - 1 ? pw - 1 : i0);
    i1 = i1 < 0 ? 0 : (i1 > pw - 1 ? pw - 1 : i1);
    j0 = j0 < 0 ? 0 : (j0 > ph - 1 ? ph - 1 : j0);
    j1 = j1 < 0 ? 0 : (j1 > ph - 1 ? ph - 1 : j1);
    for (int l = 0; l <= top; ++l) {
        const int a0 = i0 >> l, a1 = i1 >> l, b0 = j0 >> l, b1 = j1 >> l;
        if (a1 - a0 > 3 || b1 - b0 > 3) continue;
        const uint32_t mw = mip_dim((uint32_t)pw, (uint32_t)l);
        const float* img = pyr->data + mip_offset((uint32_t)pw, (uint32_t)ph, (uint32_t)l);
        for (int y = b0; y <= b1; ++y)
            for (int x = a0; x <= a1; ++x)
                if (img[(size_t)y * mw + x] < mx2) return 0;
        return 1;
    }
    return 0;
}

static int cull_draw(const orc_scene* s, const orc_camera* cam, const orc_pyramid* pyr,
                     uint32_t flags, uint32_t pass, uint32_t d, const float* eye, int* occluded) {
    *occluded = 0;
    const orc_draw* dr = &s->draws[d];
    const float* M = s->transforms + 16 * (size_t)dr->transform_index;
    const orc_primitive* prim = &s->primitives[dr->primitive_index];
    const orc_meshlet* ml = &prim->meshlets[dr->meshlet_index];
    /* worldAabbCenter (task.glsl:50) */
    float c4[4] = {ml->aabb_center[0], ml->aabb_center[1], ml->aabb_center[2], 1.0f}, wc4[4];
    m4v(M, c4, wc4);
    float wc[3] = {wc4[0], wc4[1], wc4[2]};
    /* getWorldSpaceAabbExtent (culling.h.glsl:22-29) */
    float we[3];
    const float* e = ml->aabb_extents;
    for (int j = 0; j < 3; ++j)
        we[j] = (fabsf(M[0 * 4 + j]) * e[0] + fabsf(M[1 * 4 + j]) * e[1]) + fabsf(M[2 * 4 + j]) * e[2];
    if ((flags & ORC_CULL_FRUSTUM) && !orc_frustum_visible(wc, we, (const float*)cam->frustum)) return 0;
    /* cone-culling addition: after the frustum test, before the occlusion
     * test; a double-sided material has no backface test to mirror */
    if (eye && prim->cones && !s->materials[prim->material_index].double_sided &&
        cone_culled(&prim->cones[dr->meshlet_index], M, eye))
        return 0;
    if (!(flags & ORC_CULL_OCCLUSION) || !pyr || pyr->levels == 0) return 1;
    /* projectAabb (culling.h.glsl:32-56) */
    static const float corners[8][3] = {{1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1},
                                        {1, -1, 1},  {1, 1, 1},  {-1, -1, 1}, {-1, 1, 1}};
    const float* vp = pass == 1 ? cam->prev_occlusion_vp : cam->occlusion_vp;
    float mn[3] = {1.0f, 1.0f, 1.0f}, mx[3] = {-1.0f, -1.0f, -1.0f};
    int all_front = 1;
    for (int i = 0; i < 8; ++i) {
        float p[4] = {corners[i][0] * we[0] + wc[0], corners[i][1] * we[1] + wc[1],
                      corners[i][2] * we[2] + wc[2], 1.0f};
        float clip[4];
        m4v(vp, p, clip);
        all_front &= clip[3] > 0.0f;
        /* clip.xy / clip.w and clip.z / clip.w (culling.h.glsl:49-52) as one correctly rounded
         * reciprocal of w and three products: GLSL leaves a division 2.5 ulp
         * (the perspective divide of the raster is pinned the same way) */
        float rw = 1.0f / clip[3];
        float ndx = gclamp(clip[0] * rw, -1.0f, 1.0f);
        float ndy = gclamp(clip[1] * rw, -1.0f, 1.0f);
        float q[3] = {ndx * 0.5f + 0.5f, ndy * 0.5f + 0.5f, clip[2] * rw};
        for (int k = 0; k < 3; ++k) {
            mn[k] = gmin(mn[k], q[k]);
            mx[k] = gmax(mx[k], q[k]);
        }
    }
    /* HiZ lookup (task.glsl:57-64); textureSize(level 0) = (W>>1, H>>1) */
    float width = (mx[0] - mn[0]) * (float)pyr->width;
    float height = (mx[1] - mn[1]) * (float)pyr->height;
    int lvl = hiz_level(gmax(width, height), pyr->levels);
    float cx = (mn[0] + mx[0]) * 0.5f, cy = (mn[1] + mx[1]) * 0.5f;
    uint32_t mw = mip_dim(pyr->width, (uint32_t)lvl), mh = mip_dim(pyr->height, (uint32_t)lvl);
    const float* img = pyr->data + mip_offset(pyr->width, pyr->height, (uint32_t)lvl);
    float depth = orc_min_sample(img, mw, mh, cx, cy);
    if (depth < mx[2] &&
        !((flags & ORC_CULL_OCCLUSION_FINE) && all_front &&
          fine_occluded(pyr, pyr->view_width, pyr->view_height, mn[0], mx[0], mn[1], mx[1], mx[2])))
        return 1;
    *occluded = 1;
    return 0;
}

typedef struct {
    const orc_scene* s;
    const orc_camera* cam;
    const orc_pyramid* pyr;
    uint32_t flags, pass;
    const uint32_t* cand;
    uint8_t* verdict; /* 0 culled, 1 visible, 2 occluded */
    const float* eye; /* NULL: no cone test */
} cull_ctx;

static void cull_range(void* p, int64_t b, int64_t e, int worker) {
    (void)worker;
    cull_ctx* c = (cull_ctx*)p;
    for (int64_t i = b; i < e; ++i) {
        uint32_t d = c->cand ? c->cand[i] : (uint32_t)i;
        int occ;
        int vis = cull_draw(c->s, c->cam, c->pyr, c->flags, c->pass, d, c->eye, &occ);
        c->verdict[i] = vis ? 1 : (occ ? 2 : 0);
    }
}

void orc_cull(const orc_scene* s, const orc_camera* cam, const orc_pyramid* pyr, uint32_t flags,
              uint32_t pass, const uint32_t* cand, uint32_t ncand, uint32_t* survivors, uint32_t* nsurv,
              uint32_t* rejected, uint32_t* nrej) {
    uint32_t n = cand ? ncand : s->draw_count;
    uint8_t* verdict = (uint8_t*)malloc(n ? n : 1);
    float eye[3];
    int have_eye = (flags & ORC_CULL_CONE) && eye_from_vp(cam->vp, eye);
    cull_ctx c = {s, cam, pyr, flags, pass, cand, verdict, have_eye ? eye : NULL};
    orc_parallel_for(n, cull_range, &c);
    uint32_t ns = 0, nr = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t d = cand ? cand[i] : i;
        if (verdict[i] == 1) survivors[ns++] = d;
        if (verdict[i] == 2 && rejected) rejected[nr++] = d;
    }
    free(verdict);
    *nsurv = ns;
    if (nrej) *nrej = nr;
}

/* ---------------------------------------------------------------- raster */

#define GUARD 256.0f
enum { OC_XLO = 1, OC_XHI = 2, OC_YLO = 4, OC_YHI = 8, OC_ZLO = 16, OC_ZHI = 32 };

static int outcode(const float v[4]) {
    int c = 0;
    if (v[0] < -v[3]) c |= OC_XLO;
    if (v[0] > v[3]) c |= OC_XHI;
    if (v[1] < -v[3]) c |= OC_YLO;
    if (v[1] > v[3]) c |= OC_YHI;
    if (v[2] < 0.0f) c |= OC_ZLO;
    if (v[2] > v[3]) c |= OC_ZHI;
    return c;
}

static int outside_guard(const float v[4]) {
    float g = GUARD * v[3];
    return v[0] < -g || v[0] > g || v[1] < -g || v[1] > g;
}

static float plane_dist(const float v[4], int plane) {
    switch (plane) {
        case 0: return v[3] - v[2];          /* z <= w (near, reverse-Z)  */
        case 1: return v[2];                 /* z >= 0 (far)              */
        case 2: return GUARD * v[3] - v[0];  /* x <= G w                  */
        case 3: return v[0] + GUARD * v[3];  /* x >= -G w                 */
        case 4: return GUARD * v[3] - v[1];  /* y <= G w                  */
        default: return v[1] + GUARD * v[3]; /* y >= -G w                 */
    }
}

/* Sutherland-Hodgman against one homogeneous plane. */
static int clip_poly(float in[][4], int n, float out[][4], int plane) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const float* a = in[i];
        const float* b = in[(i + 1) % n];
        float da = plane_dist(a, plane), db = plane_dist(b, plane);
        int ia = da >= 0.0f, ib = db >= 0.0f;
        if (ia) {
            memcpy(out[m], a, 16);
            ++m;
        }
        if (ia != ib) {
            float t = da / (da - db);
            for (int k = 0; k < 4; ++k) out[m][k] = a[k] + t * (b[k] - a[k]);
            ++m;
        }
    }
    return m;
}

static void atomic_max_u64(uint64_t* p, uint64_t v) {
    uint64_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

static int64_t floor_div256(int64_t a) { return a >= 0 ? a / 256 : -((-a + 255) / 256); }

/* One snapped triangle (already clipped, all w > 0). */
static void raster_snapped(int32_t X[3], int32_t Y[3], float Z[3], uint32_t id, uint32_t w, uint32_t h,
                           uint64_t* depth_id) {
    int64_t A = (int64_t)(X[1] - X[0]) * (Y[2] - Y[0]) - (int64_t)(Y[1] - Y[0]) * (X[2] - X[0]);
    if (A == 0) return;
    if (A < 0) {
        int32_t tx = X[1], ty = Y[1];
        float tz = Z[1];
        X[1] = X[2], Y[1] = Y[2], Z[1] = Z[2];
        X[2] = tx, Y[2] = ty, Z[2] = tz;
        A = -A;
    }
    int32_t minx = X[0], maxx = X[0], miny = Y[0], maxy = Y[0];
    for (int k = 1; k < 3; ++k) {
        minx = X[k] < minx ? X[k] : minx;
        maxx = X[k] > maxx ? X[k] : maxx;
        miny = Y[k] < miny ? Y[k] : miny;
        maxy = Y[k] > maxy ? Y[k] : maxy;
    }
    int64_t px0 = floor_div256((int64_t)minx - 128 + 255), px1 = floor_div256((int64_t)maxx - 128);
    int64_t py0 = floor_div256((int64_t)miny - 128 + 255), py1 = floor_div256((int64_t)maxy - 128);
    if (px0 < 0) px0 = 0;
    if (py0 < 0) py0 = 0;
    if (px1 > (int64_t)w - 1) px1 = (int64_t)w - 1;
    if (py1 > (int64_t)h - 1) py1 = (int64_t)h - 1;
    if (px0 > px1 || py0 > py1) return;
    /* top-left: an edge a->b (positive area, y down) is top or left when
     * dy < 0, or dy == 0 and dx > 0; other edges exclude their samples. */
    int64_t bias[3];
    for (int k = 0; k < 3; ++k) {
        int a = k, b = (k + 1) % 3;
        int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
        bias[k] = (dy < 0 || (dy == 0 && dx > 0)) ? 0 : 1;
    }
    /* depth plane */
    float dx1 = (float)(X[1] - X[0]), dy1 = (float)(Y[1] - Y[0]);
    float dx2 = (float)(X[2] - X[0]), dy2 = (float)(Y[2] - Y[0]);
    float af = (float)A;
    float dz1 = Z[1] - Z[0], dz2 = Z[2] - Z[0];
    float ra = 1.0f / af; /* one reciprocal of the area for both slopes */
    float pa = (dz1 * dy2 - dz2 * dy1) * ra;
    float pb = (dz2 * dx1 - dz1 * dx2) * ra;
    uint64_t lo = (uint64_t)id + 1u;
    for (int64_t py = py0; py <= py1; ++py) {
        int32_t sy = (int32_t)py * 256 + 128;
        for (int64_t px = px0; px <= px1; ++px) {
            int32_t sx = (int32_t)px * 256 + 128;
            int covered = 1;
            for (int k = 0; k < 3 && covered; ++k) {
                int a = k, b = (k + 1) % 3;
                int64_t e = (int64_t)(X[b] - X[a]) * (sy - Y[a]) - (int64_t)(Y[b] - Y[a]) * (sx - X[a]);
                covered = e >= bias[k];
            }
            if (!covered) continue;
            float z = fmaf(pa, (float)(sx - X[0]), fmaf(pb, (float)(sy - Y[0]), Z[0]));
            if (!(z > 0.0f)) z = 0.0f;
            if (z > 1.0f) z = 1.0f;
            atomic_max_u64(&depth_id[(size_t)py * w + (size_t)px], ((uint64_t)f2u(z) << 32) | lo);
        }
    }
}

void orc_raster_triangle(const float v0[4], const float v1[4], const float v2[4], uint32_t id, uint32_t w,
                         uint32_t h, uint64_t* depth_id) {
    int oc0 = outcode(v0), oc1 = outcode(v1), oc2 = outcode(v2);
    if (oc0 & oc1 & oc2) return;
    float bufa[12][4], bufb[12][4];
    memcpy(bufa[0], v0, 16);
    memcpy(bufa[1], v1, 16);
    memcpy(bufa[2], v2, 16);
    int n = 3;
    float(*cur)[4] = bufa;
    float(*nxt)[4] = bufb;
    if ((oc0 | oc1 | oc2) & (OC_ZLO | OC_ZHI)) {
        for (int plane = 0; plane < 2 && n >= 3; ++plane) {
            n = clip_poly(cur, n, nxt, plane);
            float(*t)[4] = cur;
            cur = nxt;
            nxt = t;
        }
    }
    int guard = 0;
    for (int k = 0; k < n; ++k) guard |= outside_guard(cur[k]);
    if (guard) {
        for (int plane = 2; plane < 6 && n >= 3; ++plane) {
            n = clip_poly(cur, n, nxt, plane);
            float(*t)[4] = cur;
            cur = nxt;
            nxt = t;
        }
    }
    if (n < 3) return;
    int32_t X[12], Y[12];
    float Z[12];
    const float hw = 0.5f * (float)w, hh = 0.5f * (float)h;
    for (int k = 0; k < n; ++k) {
        float cw = cur[k][3];
        if (!(cw > 0.0f)) return;
        /* perspective divide as one correctly rounded reciprocal of w and
         * three products (the division's precision is the implementation's
         * to choose, application.cpp:326-340) */
        float rw = 1.0f / cw;
        float xd = cur[k][0] * rw, yd = cur[k][1] * rw, zd = cur[k][2] * rw;
        float xf = xd * hw + hw, yf = yd * hh + hh;
        float sx = xf * 256.0f, sy = yf * 256.0f;
        if (!(fabsf(sx) < 1073741824.0f) || !(fabsf(sy) < 1073741824.0f)) return;
        X[k] = (int32_t)lrintf(sx);
        Y[k] = (int32_t)lrintf(sy);
        Z[k] = zd;
    }
    for (int k = 1; k + 1 < n; ++k) {
        int32_t tx[3] = {X[0], X[k], X[k + 1]}, ty[3] = {Y[0], Y[k], Y[k + 1]};
        float tz[3] = {Z[0], Z[k], Z[k + 1]};
        raster_snapped(tx, ty, tz, id, w, h, depth_id);
    }
}

/* Mesh shader for one draw (visbuffer.mesh.glsl:30-104) feeding the raster. */
static void raster_draw(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, uint32_t d,
                        uint64_t* depth_id) {
    const orc_draw* dr = &s->draws[d];
    const orc_primitive* prim = &s->primitives[dr->primitive_index];
    const orc_meshlet* ml = &prim->meshlets[dr->meshlet_index];
    const orc_material* mat = &s->materials[prim->material_index];
    const float* M = s->transforms + 16 * (size_t)dr->transform_index;
    float mvp[16];
    m4m(cam->vp, M, mvp);
    float clip[256][4];
    uint32_t vc = ml->vertex_count;
    /* mesh-shader output limits (mesh_common.h.glsl:36-37) */
    if (vc > 64 || ml->triangle_count > 126) return;
    for (uint32_t v = 0; v < vc; ++v) {
        uint32_t vi = prim->vertex_indices[ml->vertex_offset + v];
        const float* p = prim->vertices[vi].position;
        float p4[4] = {p[0], p[1], p[2], 1.0f};
        m4v(mvp, p4, clip[v]);
    }
    float tdet = det4(M);
    for (uint32_t t = 0; t < ml->triangle_count; ++t) {
        const uint8_t* tri = prim->primitive_indices + ml->triangle_offset + 3 * t;
        if (tri[0] >= vc || tri[1] >= vc || tri[2] >= vc) continue;
        const float* a = clip[tri[0]];
        const float* b = clip[tri[1]];
        const float* c = clip[tri[2]];
        if (!mat->double_sided) {
            float P[3] = {a[0], a[1], a[3]}, Q[3] = {b[0], b[1], b[3]}, R[3] = {c[0], c[1], c[3]};
            float det = det3(P, Q, R);
            int cull = tdet < 0.0f ? det < 0.0f : det > 0.0f;
            if (cull) continue;
        }
        orc_raster_triangle(a, b, c, (d << 7) | t, w, h, depth_id);
    }
}

typedef struct {
    const orc_scene* s;
    const orc_camera* cam;
    uint32_t w, h;
    const uint32_t* draws;
    uint64_t* depth_id;
} raster_ctx;

static void raster_range(void* p, int64_t b, int64_t e, int worker) {
    (void)worker;
    raster_ctx* c = (raster_ctx*)p;
    for (int64_t i = b; i < e; ++i) raster_draw(c->s, c->cam, c->w, c->h, c->draws[i], c->depth_id);
}

void orc_raster(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, const uint32_t* draws,
                uint32_t ndraws, uint64_t* depth_id) {
    raster_ctx c = {s, cam, w, h, draws, depth_id};
    orc_parallel_for(ndraws, raster_range, &c);
}

/* ------------------------------------------------------------------- HiZ */

typedef struct {
    const uint64_t* depth_id;
    const float* src;
    uint32_t sw, sh;  /* source size */
    float* dst;
    uint32_t dw, dh;  /* destination size (texels written) */
} hiz_ctx;

static float depth_at(const hiz_ctx* c, uint32_t x, uint32_t y) {
    if (c->depth_id) {
        uint32_t bits = (uint32_t)(c->depth_id[(size_t)y * c->sw + x] >> 32);
        float f;
        memcpy(&f, &bits, 4);
        return f;
    }
    return c->src[(size_t)y * c->sw + x];
}

static void hiz_rows(void* p, int64_t b, int64_t e, int worker) {
    (void)worker;
    hiz_ctx* c = (hiz_ctx*)p;
    for (int64_t y = b; y < e; ++y)
        for (uint32_t x = 0; x < c->dw; ++x) {
            /* hiz_reduce.comp.glsl:28 */
            float u = ((float)x + 0.5f) / (float)c->dw;
            float v = ((float)y + 0.5f) / (float)c->dh;
            int xs[2], ys[2];
            int nx = footprint_axis(u, c->sw, xs), ny = footprint_axis(v, c->sh, ys);
            float r = 0.0f;
            int first = 1;
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    float t = depth_at(c, (uint32_t)xs[i], (uint32_t)ys[j]);
                    r = first ? t : gmin(r, t);
                    first = 0;
                }
            c->dst[(size_t)y * c->dw + x] = r;
        }
}

void orc_hiz(const uint64_t* depth_id, uint32_t w, uint32_t h, float* pyramid) {
    uint32_t L = orc_pyramid_levels(w, h);
    uint32_t w0 = w >> 1, h0 = h >> 1;
    for (uint32_t i = 1; i <= L; ++i) {
        /* level i writes mip i-1 from mip i-2 (depth image for i = 1) */
        uint32_t dw = w >> i, dh = h >> i;
        float* dst = pyramid + mip_offset(w0, h0, i - 1);
        uint32_t mw = mip_dim(w0, i - 1), mh = mip_dim(h0, i - 1);
        if (dw == 0 || dh == 0) {
            /* dispatch of zero groups in the reference: never written; pinned to 0 */
            memset(dst, 0, (size_t)mw * mh * sizeof(float));
            continue;
        }
        hiz_ctx c;
        c.depth_id = i == 1 ? depth_id : NULL;
        c.src = i == 1 ? NULL : pyramid + mip_offset(w0, h0, i - 2);
        c.sw = i == 1 ? w : mip_dim(w0, i - 2);
        c.sh = i == 1 ? h : mip_dim(h0, i - 2);
        c.dst = dst;
        c.dw = dw;
        c.dh = dh;
        orc_parallel_for(dh, hiz_rows, &c);
    }
}

/* --------------------------------------------------------------- resolve */

/* fromLinear / toLinear, shaders/srgb.h.glsl:9-23. */
float orc_from_linear(float c) {
    int cutoff = c < 0.0031308f;
    float higher = 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
    float lower = c * 12.92f;
    return cutoff ? lower : higher;
}

float orc_to_linear(float c) {
    int cutoff = c < 0.04045f;
    float higher = powf((c + 0.055f) / 1.055f, 2.4f);
    float lower = c / 12.92f;
    return cutoff ? lower : higher;
}

/* Float -> UNORM8 store conversion (round to nearest even). */
uint32_t orc_unorm8(float c) {
    if (!(c > 0.0f)) return 0;
    if (c > 1.0f) c = 1.0f;
    return (uint32_t)lrintf(c * 255.0f);
}

static float half_to_float(uint16_t h) {
    uint32_t s = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 31u, m = h & 1023u, bits;
    if (e == 0) {
        if (m == 0) {
            bits = s;
        } else {
            int k = -1;
            do {
                ++k;
                m <<= 1;
            } while (!(m & 1024u));
            bits = s | ((uint32_t)(127 - 15 - k) << 23) | ((m & 1023u) << 13);
        }
    } else if (e == 31) {
        bits = s | 0x7f800000u | (m << 13);
    } else {
        bits = s | ((e + 127 - 15) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

/* Bilinear REPEAT sample with texel centres at +0.5 (the textured
 * extension's sampling rule). */
static void sample_texture(const orc_texture* t, float u, float v, float out[4]) {
    float tx = u * (float)t->width - 0.5f, ty = v * (float)t->height - 0.5f;
    float fx = floorf(tx), fy = floorf(ty);
    float ax = tx - fx, ay = ty - fy;
    int64_t x0 = (int64_t)fx, y0 = (int64_t)fy;
    int64_t W = t->width, H = t->height;
    int64_t xs[2] = {((x0 % W) + W) % W, (((x0 + 1) % W) + W) % W};
    int64_t ys[2] = {((y0 % H) + H) % H, (((y0 + 1) % H) + H) % H};
    float tex[2][2][4];
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
            size_t idx = (size_t)ys[j] * t->row_pitch + (size_t)xs[i];
            if (t->format == 0) {
                const uint8_t* p = (const uint8_t*)t->data + 4 * idx;
                for (int k = 0; k < 4; ++k) tex[j][i][k] = (float)p[k] / 255.0f;
            } else {
                const float* p = (const float*)t->data + 3 * idx;
                for (int k = 0; k < 3; ++k) tex[j][i][k] = p[k];
                tex[j][i][3] = 1.0f;
            }
        }
    for (int k = 0; k < 4; ++k) {
        float top = tex[0][0][k] + ax * (tex[0][1][k] - tex[0][0][k]);
        float bot = tex[1][0][k] + ax * (tex[1][1][k] - tex[1][0][k]);
        out[k] = top + ay * (bot - top);
    }
}

/* The visible fragment of a pixel: the triangle (drawIndex, triangle) of its
 * id, its vertices in clip space (position of visbuffer.mesh.glsl:57-63) and
 * the perspective-correct barycentrics of the pixel centre. */
typedef struct {
    const orc_vertex* vx[3];
    const orc_material* mat;
    const float* M;
    float c[3][4];
    float l[3];
} orc_frag;

static void frag_setup(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, uint32_t px, uint32_t py,
                       uint32_t id, orc_frag* f) {
    uint32_t d = id >> 7, t = id & 127u;
    const orc_draw* dr = &s->draws[d];
    const orc_primitive* prim = &s->primitives[dr->primitive_index];
    const orc_meshlet* ml = &prim->meshlets[dr->meshlet_index];
    f->mat = &s->materials[prim->material_index];
    f->M = s->transforms + 16 * (size_t)dr->transform_index;
    float mvp[16];
    m4m(cam->vp, f->M, mvp);
    const uint8_t* tri = prim->primitive_indices + ml->triangle_offset + 3 * t;
    for (int k = 0; k < 3; ++k) {
        f->vx[k] = &prim->vertices[prim->vertex_indices[ml->vertex_offset + tri[k]]];
        float p4[4] = {f->vx[k]->position[0], f->vx[k]->position[1], f->vx[k]->position[2], 1.0f};
        m4v(mvp, p4, f->c[k]);
    }
    /* clip-space weights whose point projects to the pixel centre ~ a x b */
    float nx = (((float)px + 0.5f) / (float)w) * 2.0f - 1.0f;
    float ny = (((float)py + 0.5f) / (float)h) * 2.0f - 1.0f;
    float a[3], b[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = f->c[k][0] - nx * f->c[k][3];
        b[k] = f->c[k][1] - ny * f->c[k][3];
    }
    float* l = f->l;
    l[0] = a[1] * b[2] - a[2] * b[1];
    l[1] = a[2] * b[0] - a[0] * b[2];
    l[2] = a[0] * b[1] - a[1] * b[0];
    float sum = (l[0] + l[1]) + l[2];
    if (sum != 0.0f) {
        for (int k = 0; k < 3; ++k) l[k] = l[k] / sum;
    } else {
        l[0] = l[1] = l[2] = 1.0f / 3.0f;
    }
}

static float interp3(const float l[3], float v0, float v1, float v2) { return (l[0] * v0 + l[1] * v1) + l[2] * v2; }

/* Textured resolve of one pixel (extension): vertex colour, transformUv
 * (mesh_common.h.glsl:129-135), albedo texture through toLinear, as in the
 * commented-out visbuffer.frag.glsl:29-34. */
static void resolve_textured_px(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, uint32_t px,
                                uint32_t py, uint32_t id, float out[4]) {
    orc_frag f;
    frag_setup(s, cam, w, h, px, py, id, &f);
    const orc_material* mat = f.mat;
    const float* l = f.l;
    float col[4], uv[2];
    for (int k = 0; k < 4; ++k)
        col[k] = interp3(l, (float)f.vx[0]->color[k] / 255.0f, (float)f.vx[1]->color[k] / 255.0f,
                         (float)f.vx[2]->color[k] / 255.0f);
    for (int k = 0; k < 2; ++k)
        uv[k] = interp3(l, half_to_float(f.vx[0]->uv[k]), half_to_float(f.vx[1]->uv[k]), half_to_float(f.vx[2]->uv[k]));
    float sampled[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    if (mat->albedo_index != 0xFFFFFFFFu && mat->albedo_index < s->texture_count) {
        float cs = cosf(mat->uv_rotation), sn = sinf(mat->uv_rotation);
        float ru = cs * uv[0] + sn * uv[1], rv = -sn * uv[0] + cs * uv[1];
        float tu = ru * mat->uv_scale[0] + mat->uv_offset[0];
        float tv = rv * mat->uv_scale[1] + mat->uv_offset[1];
        const orc_texture* tex = &s->textures[mat->albedo_index];
        sample_texture(tex, tu, tv, sampled);
        if (tex->format == 0)
            for (int k = 0; k < 3; ++k) sampled[k] = orc_to_linear(sampled[k]);
    }
    for (int k = 0; k < 4; ++k) out[k] = col[k] * mat->albedo_factor[k] * sampled[k];
}

/* IEEE 754 binary32 -> binary16, round to nearest, ties to even; overflow
 * rounds to infinity, NaN becomes the quiet NaN 0x7E00 with its sign. */
uint16_t orc_half_rn(float v) {
    uint32_t x = f2u(v);
    uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7FFFFFFFu;
    if (ax > 0x7F800000u) return (uint16_t)(sign | 0x7E00u);
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u); /* >= 65520: past the last tie */
    if (ax < 0x38800000u) {                                    /* below 2^-14: subnormal half */
        if (ax <= 0x33000000u) return (uint16_t)sign;         /* <= 2^-25 rounds to zero (tie to even) */
        uint32_t e = ax >> 23, m = (ax & 0x7FFFFFu) | 0x800000u;
        uint32_t shift = 126u - e; /* value / 2^-24 = m >> shift, shift in [14, 24] */
        uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (q & 1u))) ++q;
        return (uint16_t)(sign | q);
    }
    uint32_t r = ax - 0x38000000u; /* rebias the exponent from 127 to 15 */
    uint32_t q = r >> 13, rem = r & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ++q; /* a carry moves into the exponent */
    return (uint16_t)(sign | q);
}

/* Motion vectors (visbuffer.frag.glsl:38) from the varyings position and
 * prevPosition (visbuffer.mesh.glsl:44-64): viewProjection * M * vertex and
 * prevViewProjection * M * vertex with the node's current transform M (the
 * reference has no previous-frame transforms), interpolated with the
 * fragment's barycentrics, then
 *   mv = (prev.xy / prev.w * 0.5 - 0.5) - (pos.xy / pos.w * 0.5 - 0.5)
 * stored as two binary16 (R16G16_SFLOAT, application.cpp:250-270), x in the
 * low half; the attachment is cleared to 0 (application.cpp:786-797). */
static uint32_t motion_px(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, uint32_t px,
                          uint32_t py, uint32_t id) {
    orc_frag f;
    frag_setup(s, cam, w, h, px, py, id, &f);
    float pmvp[16], p[3][4];
    m4m(cam->prev_vp, f.M, pmvp);
    for (int k = 0; k < 3; ++k) {
        float p4[4] = {f.vx[k]->position[0], f.vx[k]->position[1], f.vx[k]->position[2], 1.0f};
        m4v(pmvp, p4, p[k]);
    }
    float cw = interp3(f.l, f.c[0][3], f.c[1][3], f.c[2][3]);
    float pw = interp3(f.l, p[0][3], p[1][3], p[2][3]);
    uint32_t out = 0;
    for (int j = 0; j < 2; ++j) {
        float cj = interp3(f.l, f.c[0][j], f.c[1][j], f.c[2][j]);
        float pj = interp3(f.l, p[0][j], p[1][j], p[2][j]);
        float cur = (cj / cw) * 0.5f - 0.5f;
        float prev = (pj / pw) * 0.5f - 0.5f;
        out |= (uint32_t)orc_half_rn(prev - cur) << (16 * j);
    }
    return out;
}

typedef struct {
    const orc_scene* s;
    const orc_camera* cam;
    uint32_t w, h;
    const uint64_t* depth_id;
    uint32_t* motion;
} motion_ctx;

static void motion_rows(void* p, int64_t b, int64_t e, int worker) {
    (void)worker;
    motion_ctx* c = (motion_ctx*)p;
    for (int64_t y = b; y < e; ++y)
        for (uint32_t x = 0; x < c->w; ++x) {
            size_t i = (size_t)y * c->w + x;
            uint32_t lo = (uint32_t)c->depth_id[i];
            c->motion[i] = lo ? motion_px(c->s, c->cam, c->w, c->h, x, (uint32_t)y, lo - 1u) : 0u;
        }
}

void orc_motion(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, const uint64_t* depth_id,
                uint32_t* motion) {
    motion_ctx c = {s, cam, w, h, depth_id, motion};
    orc_parallel_for(h, motion_rows, &c);
}

typedef struct {
    const orc_scene* s;
    const orc_camera* cam;
    uint32_t w, h;
    const uint64_t* depth_id;
    uint32_t textured;
    uint32_t *ids, *rgba;
} resolve_ctx;

static void resolve_rows(void* p, int64_t b, int64_t e, int worker) {
    (void)worker;
    resolve_ctx* c = (resolve_ctx*)p;
    for (int64_t y = b; y < e; ++y)
        for (uint32_t x = 0; x < c->w; ++x) {
            size_t i = (size_t)y * c->w + x;
            uint32_t lo = (uint32_t)c->depth_id[i];
            uint32_t id = lo ? lo - 1u : 0xFFFFFFFFu;
            if (c->ids) c->ids[i] = id;
            if (!c->rgba) continue;
            /* visbuffer_resolve.comp.glsl:24-27: clear, then leave empty pixels at 0 */
            if (id == 0xFFFFFFFFu) {
                c->rgba[i] = 0;
                continue;
            }
            float lin[4];
            if (c->textured) {
                resolve_textured_px(c->s, c->cam, c->w, c->h, x, (uint32_t)y, id, lin);
            } else {
                const orc_draw* dr = &c->s->draws[id >> 7];
                const orc_primitive* prim = &c->s->primitives[dr->primitive_index];
                const orc_material* mat = &c->s->materials[prim->material_index];
                for (int k = 0; k < 4; ++k) lin[k] = mat->albedo_factor[k];
            }
            uint32_t r = orc_unorm8(orc_from_linear(lin[0]));
            uint32_t g = orc_unorm8(orc_from_linear(lin[1]));
            uint32_t bl = orc_unorm8(orc_from_linear(lin[2]));
            uint32_t a = orc_unorm8(lin[3]);
            c->rgba[i] = r | (g << 8) | (bl << 16) | (a << 24);
        }
}

void orc_resolve(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, const uint64_t* depth_id,
                 uint32_t textured, uint32_t* ids, uint32_t* rgba) {
    resolve_ctx c = {s, cam, w, h, depth_id, textured, ids, rgba};
    orc_parallel_for(h, resolve_rows, &c);
}

/* ----------------------------------------------------------------- frame */

/* Same pass structure as vkgv_frame: clear; pass-1 cull against the
 * previous pyramid; raster; with two-pass culling: pyramid from this depth,
 * pass-2 re-test of the occlusion rejects, raster; final pyramid; resolve. */
void orc_frame(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, const orc_pyramid* prev,
               uint32_t flags, uint64_t* depth_id, uint32_t* ids, uint32_t* rgba, float* pyramid_out,
               uint32_t* survivors, uint32_t* nsurv) {
    uint32_t D = s->draw_count;
    memset(depth_id, 0, (size_t)w * h * sizeof(uint64_t));
    uint32_t* rej = (uint32_t*)malloc((size_t)(D ? D : 1) * sizeof(uint32_t));
    uint32_t ns1 = 0, nr = 0;
    orc_cull(s, cam, prev, flags, 1, NULL, 0, survivors, &ns1, rej, &nr);
    orc_raster(s, cam, w, h, survivors, ns1, depth_id);
    uint32_t total = ns1;
    int two = (flags & ORC_CULL_TWO_PASS) && (flags & ORC_CULL_OCCLUSION) && prev && prev->levels > 0 &&
              pyramid_out;
    if (two) {
        orc_hiz(depth_id, w, h, pyramid_out);
        orc_pyramid cur = {pyramid_out, w >> 1, h >> 1, orc_pyramid_levels(w, h), w, h};
        uint32_t ns2 = 0;
        orc_cull(s, cam, &cur, flags, 2, rej, nr, survivors + ns1, &ns2, NULL, NULL);
        orc_raster(s, cam, w, h, survivors + ns1, ns2, depth_id);
        total += ns2;
    }
    if ((flags & ORC_BUILD_PYRAMID) && pyramid_out) orc_hiz(depth_id, w, h, pyramid_out);
    if (ids || rgba) orc_resolve(s, cam, w, h, depth_id, (flags & ORC_RESOLVE_TEXTURED) ? 1u : 0u, ids, rgba);
    free(rej);
    *nsurv = total;
}

/* ------------------------------------------------- adjoint (float64) */

static int wrapi(int64_t i, int64_t n) {
    int64_t r = i % n;
    return (int)(r < 0 ? r + n : r);
}

/* Forward shading and its exact derivative in float64 at fixed visibility
 * (the differentiable form of the commented-out visbuffer.frag.glsl:29-34;
 * transformUv as mesh_common.h.glsl:129-135). */
double orc_diff_f64(const orc_diff_scene* s, const float vpf[16], uint32_t w, uint32_t h, const uint32_t* ids,
                    const float* target, double scale, double* rgb_out, double* gpos, double* gcol, double* gtex,
                    int32_t* cells) {
    return orc_diff_f64_frozen(s, vpf, w, h, ids, target, scale, rgb_out, gpos, gcol, gtex, cells, NULL, NULL);
}

/* As orc_diff_f64; with `freeze` (2 per pixel, as `cells` reports them) each
 * covered pixel samples the bilinear patch of its frozen cell, extended
 * linearly past the cell's texel centres: the smooth piece of the filtered
 * texture that holds the pixel's sample at the frozen parameters, whose
 * derivative is the gradient there.  A finite difference of this loss is
 * free of the derivative jumps at texel centres. */
double orc_diff_f64_frozen(const orc_diff_scene* s, const float vpf[16], uint32_t w, uint32_t h, const uint32_t* ids,
                           const float* target, double scale, double* rgb_out, double* gpos, double* gcol,
                           double* gtex, int32_t* cells, const int32_t* freeze, double* margin) {
    double vp[16];
    for (int k = 0; k < 16; ++k) vp[k] = vpf[k];
    const double cs = cos(s->uv_rotation), sn = sin(s->uv_rotation);
    double loss = 0.0;
    for (uint32_t py = 0; py < h; ++py)
        for (uint32_t px = 0; px < w; ++px) {
            const size_t p = (size_t)py * w + px;
            double tg[3] = {0, 0, 0};
            if (target)
                for (int j = 0; j < 3; ++j) tg[j] = target[3 * p + j];
            const uint32_t id = ids[p];
            double shade[3] = {0, 0, 0};
            if (cells) cells[2 * p] = cells[2 * p + 1] = INT32_MIN;
            if (margin) margin[p] = -1.0;
            if (id == 0xFFFFFFFFu) {
                if (rgb_out)
                    for (int j = 0; j < 3; ++j) rgb_out[3 * p + j] = 0.0;
                for (int j = 0; j < 3; ++j) loss += scale * tg[j] * tg[j];
                continue;
            }
            const orc_meshlet* ml = &s->meshlets[id >> 7];
            const uint8_t* tri = s->tri_indices + ml->triangle_offset + 3 * (id & 127u);
            uint32_t vi[3];
            double c[3][4];
            for (int k = 0; k < 3; ++k) {
                vi[k] = s->vertex_indices[ml->vertex_offset + tri[k]];
                const double* q = s->positions + 3 * (size_t)vi[k];
                for (int r = 0; r < 4; ++r) c[k][r] = vp[0 * 4 + r] * q[0] + vp[1 * 4 + r] * q[1] + vp[2 * 4 + r] * q[2] + vp[3 * 4 + r];
            }
            /* the sample point is the fp32 NDC of the pixel centre (the
             * point the GPU evaluates), then carried in double */
            const double nx = (double)(((float)px + 0.5f) / (float)w * 2.0f - 1.0f);
            const double ny = (double)(((float)py + 0.5f) / (float)h * 2.0f - 1.0f);
            double a[3], b[3];
            for (int k = 0; k < 3; ++k) {
                a[k] = c[k][0] - nx * c[k][3];
                b[k] = c[k][1] - ny * c[k][3];
            }
            const double l[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            const double sum = l[0] + l[1] + l[2];
            if (sum == 0.0) {
                if (rgb_out)
                    for (int j = 0; j < 3; ++j) rgb_out[3 * p + j] = 0.0;
                for (int j = 0; j < 3; ++j) loss += scale * tg[j] * tg[j];
                continue;
            }
            const double lam[3] = {l[0] / sum, l[1] / sum, l[2] / sum};
            double col[3], uv[2];
            for (int j = 0; j < 3; ++j)
                col[j] = lam[0] * s->colors[3 * (size_t)vi[0] + j] + lam[1] * s->colors[3 * (size_t)vi[1] + j] +
                         lam[2] * s->colors[3 * (size_t)vi[2] + j];
            for (int j = 0; j < 2; ++j)
                uv[j] = lam[0] * s->uvs[2 * (size_t)vi[0] + j] + lam[1] * s->uvs[2 * (size_t)vi[1] + j] +
                        lam[2] * s->uvs[2 * (size_t)vi[2] + j];
            const double ru = cs * uv[0] + sn * uv[1], rv = -sn * uv[0] + cs * uv[1];
            const double tu = ru * s->uv_scale[0] + s->uv_offset[0], tv = rv * s->uv_scale[1] + s->uv_offset[1];
            const double tx = tu * s->tex_w - 0.5, ty = tv * s->tex_h - 0.5;
            double fx = floor(tx), fy = floor(ty);
            if (margin) {
                /* texels from the sample to the nearest texel-centre line,
                 * where the bilinear derivative jumps */
                const double mx = fmin(tx - fx, fx + 1.0 - tx), my = fmin(ty - fy, fy + 1.0 - ty);
                margin[p] = fmin(mx, my);
            }
            if (freeze && freeze[2 * p] != INT32_MIN) {
                fx = (double)freeze[2 * p];
                fy = (double)freeze[2 * p + 1];
            }
            const double ax = tx - fx, ay = ty - fy;
            if (cells) {
                cells[2 * p] = (int32_t)fx;
                cells[2 * p + 1] = (int32_t)fy;
            }
            const int x0 = wrapi((int64_t)fx, s->tex_w), x1 = wrapi((int64_t)fx + 1, s->tex_w);
            const int y0 = wrapi((int64_t)fy, s->tex_h), y1 = wrapi((int64_t)fy + 1, s->tex_h);
            const size_t i00 = 3 * ((size_t)y0 * s->tex_w + x0), i01 = 3 * ((size_t)y0 * s->tex_w + x1);
            const size_t i10 = 3 * ((size_t)y1 * s->tex_w + x0), i11 = 3 * ((size_t)y1 * s->tex_w + x1);
            const double* T = s->texture;
            double tex[3];
            for (int j = 0; j < 3; ++j) {
                const double top = T[i00 + j] + ax * (T[i01 + j] - T[i00 + j]);
                const double bot = T[i10 + j] + ax * (T[i11 + j] - T[i10 + j]);
                tex[j] = top + ay * (bot - top);
                shade[j] = col[j] * s->albedo[j] * tex[j];
            }
            if (rgb_out)
                for (int j = 0; j < 3; ++j) rgb_out[3 * p + j] = shade[j];
            double g[3], dcol[3], dtex[3];
            for (int j = 0; j < 3; ++j) {
                const double r = shade[j] - tg[j];
                loss += scale * r * r;
                g[j] = 2.0 * scale * r;
                dcol[j] = g[j] * s->albedo[j] * tex[j];
                dtex[j] = g[j] * col[j] * s->albedo[j];
            }
            if (gtex) {
                const double w00 = (1 - ax) * (1 - ay), w01 = ax * (1 - ay), w10 = (1 - ax) * ay, w11 = ax * ay;
                for (int j = 0; j < 3; ++j) {
                    gtex[i00 + j] += dtex[j] * w00;
                    gtex[i01 + j] += dtex[j] * w01;
                    gtex[i10 + j] += dtex[j] * w10;
                    gtex[i11 + j] += dtex[j] * w11;
                }
            }
            double dtu = 0, dtv = 0;
            for (int j = 0; j < 3; ++j) {
                dtu += dtex[j] * ((1 - ay) * (T[i01 + j] - T[i00 + j]) + ay * (T[i11 + j] - T[i10 + j]));
                dtv += dtex[j] * ((1 - ax) * (T[i10 + j] - T[i00 + j]) + ax * (T[i11 + j] - T[i01 + j]));
            }
            dtu *= s->tex_w;
            dtv *= s->tex_h;
            const double dru = dtu * s->uv_scale[0], drv = dtv * s->uv_scale[1];
            const double du = cs * dru - sn * drv, dv = sn * dru + cs * drv;
            double dlam[3];
            for (int k = 0; k < 3; ++k) {
                dlam[k] = du * s->uvs[2 * (size_t)vi[k]] + dv * s->uvs[2 * (size_t)vi[k] + 1];
                for (int j = 0; j < 3; ++j) {
                    dlam[k] += dcol[j] * s->colors[3 * (size_t)vi[k] + j];
                    if (gcol) gcol[3 * (size_t)vi[k] + j] += dcol[j] * lam[k];
                }
            }
            if (!gpos) continue;
            const double dot = lam[0] * dlam[0] + lam[1] * dlam[1] + lam[2] * dlam[2];
            const double dl[3] = {(dlam[0] - dot) / sum, (dlam[1] - dot) / sum, (dlam[2] - dot) / sum};
            const double da[3] = {b[1] * dl[2] - b[2] * dl[1], b[2] * dl[0] - b[0] * dl[2], b[0] * dl[1] - b[1] * dl[0]};
            const double db[3] = {dl[1] * a[2] - dl[2] * a[1], dl[2] * a[0] - dl[0] * a[2], dl[0] * a[1] - dl[1] * a[0]};
            for (int k = 0; k < 3; ++k) {
                const double dx = da[k], dy = db[k], dw = -nx * da[k] - ny * db[k];
                for (int q = 0; q < 3; ++q)
                    gpos[3 * (size_t)vi[k] + q] += vp[q * 4 + 0] * dx + vp[q * 4 + 1] * dy + vp[q * 4 + 3] * dw;
            }
        }
    return loss;
}
