/*
 * world.c: CPU restatement of vk_gltf_viewer's per-frame world update
 * (src/vk_gltf_viewer/world.cpp:187-345) and its animation sampler
 * (include/vk_gltf_viewer/assets.hpp:51-113).  TEST INFRASTRUCTURE ONLY: the
 * parity tests and the benchmark's CPU leg call it as the checker.
 *
 * The traversal follows the reference literally: a recursive depth-first walk
 * from each scene root (World::iterateNode, world.cpp:187-224) that, at every
 * node, loops over every channel of every animation to find those that target
 * it (world.cpp:192-213), composes the parent matrix with the animated TRS,
 * hands the node to the callback (a transform index for nodes with a mesh,
 * world.cpp:242-262 and 299-311) and then recurses into the children.
 *
 * The vector arithmetic that the reference takes from fastgltf (absent from
 * the reference tree, version unpinned) is restated from the glTF 2.0
 * specification's animation appendix with a pinned operation order:
 *   lerp   (1 - t) * a + t * b
 *   slerp  in float: b' = -b when dot(a, b) < 0; sin(theta/2) = |a - b'| / 2,
 *          cos(theta/2) = |a + b'| / 2, sin(theta/4) = sin(theta/2) /
 *          sqrt(2 (1 + cos(theta/2))), theta = 4 asin(sin(theta/4)) by the
 *          asin power series (10 terms), weights sin((1-t) theta) / sin(theta)
 *          and sin(t theta) / sin(theta) by the sine Taylor series (8 terms;
 *          linear weights below theta = 1e-6)
 *   cubic  the Hermite form of assets.hpp:93-108 with t^2 = t*t, t^3 = t^2*t
 *          (the reference calls powf), rotation normalised by v / |v|
 *   node   parent * (T * R * S) with the rotation matrix of the unit
 *          quaternion (the reference's translate/rotate/scale chain,
 *          world.cpp:217, associated as one local matrix)
 * The parity of those steps with the reference's own execution is therefore
 * unpinned; the traversal order, the sampler's boundary and looping rules and
 * the draw and transform numbering are the reference's.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* (-1)^k / (2k+1)!, k = 0..7, rounded to float */
static const float kSin[8] = {0x1.000000p+0f,  -0x1.555556p-3f, 0x1.111112p-7f,  -0x1.a01a02p-13f,
                              0x1.71de3ap-19f, -0x1.ae6456p-26f, 0x1.612462p-33f, -0x1.ae7f3ep-41f};
/* C(2n, n) / (4^n (2n + 1)), n = 0..9, rounded to float */
static const float kAsin[10] = {0x1.000000p+0f, 0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f, 0x1.f1c71cp-6f,
                                0x1.6e8ba2p-6f, 0x1.1c4ec4p-6f, 0x1.c9999ap-7f, 0x1.7a8788p-7f, 0x1.3fde50p-7f};

float orc_sin_series(float x) {
    float u = x * x, p = kSin[7];
    for (int k = 6; k >= 0; --k) p = p * u + kSin[k];
    return x * p;
}

float orc_asin_series(float z) {
    float u = z * z, p = kAsin[9];
    for (int k = 8; k >= 0; --k) p = p * u + kAsin[k];
    return z * p;
}

void orc_slerp(const float a[4], const float b[4], float t, float out[4]) {
    float A[4], B[4];
    for (int k = 0; k < 4; ++k) {
        A[k] = a[k];
        B[k] = b[k];
    }
    float d = ((A[0] * B[0] + A[1] * B[1]) + A[2] * B[2]) + A[3] * B[3];
    if (d < 0.0f)
        for (int k = 0; k < 4; ++k) B[k] = -B[k];
    float sd = 0.0f, sp = 0.0f;
    for (int k = 0; k < 4; ++k) {
        float m = A[k] - B[k], p = A[k] + B[k];
        sd = sd + m * m;
        sp = sp + p * p;
    }
    float s = 0.5f * sqrtf(sd), c = 0.5f * sqrtf(sp);
    float z = s / sqrtf(2.0f * (1.0f + c));
    float theta = 4.0f * orc_asin_series(z);
    float w0 = 1.0f - t, w1 = t;
    if (theta >= 1e-6f) {
        float sn = orc_sin_series(theta);
        if (sn != 0.0f) {
            w0 = orc_sin_series((1.0f - t) * theta) / sn;
            w1 = orc_sin_series(t * theta) / sn;
        }
    }
    for (int k = 0; k < 4; ++k) out[k] = w0 * A[k] + w1 * B[k];
}

/* AnimationSampler::sample (assets.hpp:56-113). */
void orc_anim_sample(const orc_anim_sampler* S, float time, uint32_t path, float out[4]) {
    const float* in = S->input;
    const float* val = S->output;
    uint32_t n = S->input_count, cc = S->components;
    int cubic = S->interpolation == ORC_INTERP_CUBICSPLINE;
    float tt = fmodf(time, in[n - 1]); /* assets.hpp:61, loops the animation */
    uint32_t lo = 0, hi = n;            /* std::lower_bound (assets.hpp:63) */
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (in[mid] < tt)
            lo = mid + 1;
        else
            hi = mid;
    }
    const float* src;
    if (lo == 0) { /* assets.hpp:64-68 */
        src = val + (cubic ? 1u : 0u) * cc;
    } else if (lo == n) { /* assets.hpp:69-73 */
        src = val + (cubic ? S->output_count - 2u : S->output_count - 1u) * cc;
    } else {
        uint32_t i = lo;
        float t = (tt - in[i - 1]) / (in[i] - in[i - 1]); /* assets.hpp:76 */
        if (S->interpolation == ORC_INTERP_STEP) {         /* assets.hpp:80-81 */
            src = val + (i - 1) * cc;
        } else if (S->interpolation == ORC_INTERP_LINEAR) { /* assets.hpp:82-91 */
            const float* a = val + (i - 1) * cc;
            const float* b = val + i * cc;
            if (path == ORC_PATH_ROTATION) {
                orc_slerp(a, b, t, out);
            } else {
                float u = 1.0f - t;
                for (uint32_t k = 0; k < cc; ++k) out[k] = u * a[k] + t * b[k];
            }
            return;
        } else { /* CUBICSPLINE, assets.hpp:93-108 */
            float t2 = t * t, t3 = t2 * t;
            float dt = in[i] - in[i - 1];
            float h00 = (2.0f * t3 - 3.0f * t2) + 1.0f;
            float h10 = (t3 - 2.0f * t2) + t;
            float h01 = -2.0f * t3 + 3.0f * t2;
            float h11 = t3 - t2;
            const float* p0 = val + (3 * (i - 1) + 1) * cc;
            const float* m0 = val + (3 * (i - 1) + 2) * cc;
            const float* p1 = val + (3 * i + 1) * cc;
            const float* m1 = val + (3 * i + 0) * cc;
            for (uint32_t k = 0; k < cc; ++k)
                out[k] = ((p0[k] * h00 + (m0[k] * h10) * dt) + p1[k] * h01) + (m1[k] * h11) * dt;
            if (path == ORC_PATH_ROTATION) {
                float len = sqrtf(((out[0] * out[0] + out[1] * out[1]) + out[2] * out[2]) + out[3] * out[3]);
                for (int k = 0; k < 4; ++k) out[k] = out[k] / len;
            }
            return;
        }
    }
    for (uint32_t k = 0; k < cc; ++k) out[k] = src[k];
}

/* T * R * S, column-major. */
void orc_trs_matrix(const float t[3], const float q[4], const float s[3], float m[16]) {
    float x = q[0], y = q[1], z = q[2], w = q[3];
    float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
    float wx = w * x, wy = w * y, wz = w * z;
    float r[9] = {1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy),
                  2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx),
                  2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy)};
    for (int c = 0; c < 3; ++c) {
        for (int j = 0; j < 3; ++j) m[4 * c + j] = r[3 * c + j] * s[c];
        m[4 * c + 3] = 0.0f;
    }
    m[12] = t[0];
    m[13] = t[1];
    m[14] = t[2];
    m[15] = 1.0f;
}

/* r = a * b (column-major), sums ((a0 b0 + a1 b1) + a2 b2) + a3 b3. */
static void mat_mul(const float* a, const float* b, float* r) {
    for (int c = 0; c < 4; ++c)
        for (int j = 0; j < 4; ++j)
            r[c * 4 + j] = ((a[0 * 4 + j] * b[c * 4 + 0] + a[1 * 4 + j] * b[c * 4 + 1]) + a[2 * 4 + j] * b[c * 4 + 2]) +
                           a[3 * 4 + j] * b[c * 4 + 3];
}

typedef struct {
    const orc_world* w;
    float time;
    int with_matrices;
    float* transforms; /* 16 per slot, or NULL */
    uint32_t* draws;   /* 3 words per draw, or NULL */
    uint64_t draw_capacity, draw_count;
    uint32_t transform_capacity, transform_count;
    int error;
} walk_ctx;

/* The callback of world.cpp:242-262 (draws) and 299-311 (transforms). */
static void visit(walk_ctx* c, const orc_node* node, const float* matrix) {
    if (node->mesh_index == 0xFFFFFFFFu) return;
    uint32_t transform_index = c->transform_count++;
    if (c->transforms && transform_index < c->transform_capacity)
        memcpy(c->transforms + 16 * (size_t)transform_index, matrix, 16 * sizeof(float));
    const orc_world* w = c->w;
    for (uint32_t i = w->mesh_offsets[node->mesh_index]; i < w->mesh_offsets[node->mesh_index + 1]; ++i) {
        uint32_t prim = w->mesh_primitives[i];
        for (uint32_t m = 0; m < w->primitive_meshlet_counts[prim]; ++m) {
            uint64_t d = c->draw_count++;
            if (c->draws && d < c->draw_capacity) {
                c->draws[3 * d + 0] = prim;
                c->draws[3 * d + 1] = m;
                c->draws[3 * d + 2] = transform_index;
            }
        }
    }
}

/* World::iterateNode (world.cpp:187-224). */
static void iterate_node(walk_ctx* c, uint32_t index, const float parent[16], uint32_t depth) {
    if (depth >= 64) {
        c->error = 1;
        return;
    }
    const orc_world* w = c->w;
    const orc_node* node = &w->nodes[index];
    float matrix[16];
    if (c->with_matrices) {
        float t[3] = {node->translation[0], node->translation[1], node->translation[2]};
        float q[4] = {node->rotation[0], node->rotation[1], node->rotation[2], node->rotation[3]};
        float s[3] = {node->scale[0], node->scale[1], node->scale[2]};
        for (uint32_t ch = 0; ch < w->channel_count; ++ch) {
            const orc_anim_channel* a = &w->channels[ch];
            if (a->node != index) continue;
            float v[4];
            if (a->path == ORC_PATH_TRANSLATION) {
                orc_anim_sample(&w->samplers[a->sampler], c->time, a->path, v);
                t[0] = v[0], t[1] = v[1], t[2] = v[2];
            } else if (a->path == ORC_PATH_SCALE) {
                orc_anim_sample(&w->samplers[a->sampler], c->time, a->path, v);
                s[0] = v[0], s[1] = v[1], s[2] = v[2];
            } else if (a->path == ORC_PATH_ROTATION) {
                orc_anim_sample(&w->samplers[a->sampler], c->time, a->path, v);
                q[0] = v[0], q[1] = v[1], q[2] = v[2], q[3] = v[3];
            }
        }
        float local[16];
        orc_trs_matrix(t, q, s, local);
        mat_mul(parent, local, matrix);
    } else {
        memset(matrix, 0, sizeof(matrix));
    }
    visit(c, node, matrix);
    for (uint32_t k = 0; k < node->child_count && !c->error; ++k)
        iterate_node(c, w->children[node->first_child + k], matrix, depth + 1);
}

static void walk(walk_ctx* c) {
    static const float identity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (uint32_t r = 0; r < c->w->root_count && !c->error; ++r) iterate_node(c, c->w->roots[r], identity, 0);
}

int64_t orc_world_transforms(const orc_world* w, float animation_time, float* transforms, uint32_t capacity) {
    walk_ctx c;
    memset(&c, 0, sizeof(c));
    c.w = w;
    c.time = animation_time;
    c.with_matrices = 1;
    c.transforms = transforms;
    c.transform_capacity = capacity;
    walk(&c);
    return c.error ? -1 : (int64_t)c.transform_count;
}

int64_t orc_world_draws(const orc_world* w, uint32_t* draws, uint64_t capacity) {
    walk_ctx c;
    memset(&c, 0, sizeof(c));
    c.w = w;
    c.draws = draws;
    c.draw_capacity = capacity;
    walk(&c);
    return c.error ? -1 : (int64_t)c.draw_count;
}
