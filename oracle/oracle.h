/*
 * oracle.h — CPU restatement of vk_gltf_viewer's meshlet visibility-buffer
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark call it as the checker.  The product
 * library never links or calls it.
 *
 * Parity status: the reference renderer cannot execute here (it needs a
 * Vulkan 1.3 mesh-shader device and glslangValidator; no graphics stack
 * exists on either machine), so the restatement is pinned by hand-derived
 * known-answer cases (tests/golden/kat_*.json) and by the reference's
 * constants, not by reference output.  Parity with the reference's own
 * execution is therefore unpinned beyond those cases.
 *
 * Every function follows the reference file:line named in its comment.  The
 * parts the reference leaves to the Vulkan implementation (rasterisation
 * rules, depth interpolation, min-reduction sampler footprint, clipping)
 * are pinned as documented in oracle.c and implemented identically by the
 * CUDA kernels.
 */
#ifndef VKGV_ORACLE_H
#define VKGV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layout restatements (shaders/mesh_common.h.glsl:20-126, scalar layout). */
typedef struct orc_meshlet {
    uint32_t vertex_offset, triangle_offset;
    uint8_t vertex_count, triangle_count, pad_[2];
    float aabb_extents[3], aabb_center[3];
} orc_meshlet; /* 36 B */

typedef struct orc_vertex {
    float position[3];
    uint8_t color[4];
    uint8_t normal[3];
    uint8_t pad_;
    uint16_t uv[2];
} orc_vertex; /* 24 B */

typedef struct orc_draw {
    uint32_t primitive_index, meshlet_index, transform_index;
} orc_draw; /* 12 B */

typedef struct orc_material {
    float albedo_factor[4];
    uint32_t albedo_index;
    float uv_offset[2], uv_scale[2], uv_rotation, alpha_cutoff;
    uint32_t double_sided;
} orc_material; /* 48 B */

typedef struct orc_camera {
    float prev_vp[16], prev_occlusion_vp[16], vp[16], occlusion_vp[16];
    float frustum[6][4];
} orc_camera; /* 352 B */

/* Meshlet normal cone (object space) used by the cone-culling addition. */
typedef struct orc_cone {
    float center[3], radius, axis[3], cutoff;
} orc_cone; /* 32 B */

/* A primitive with host pointers in place of the device addresses. */
typedef struct orc_primitive {
    const uint32_t* vertex_indices;
    const uint8_t* primitive_indices;
    const orc_vertex* vertices;
    const orc_meshlet* meshlets;
    float aabb_extents[3], aabb_center[3];
    uint32_t meshlet_count, material_index;
    const orc_cone* cones; /* NULL: no cone culling for this primitive */
} orc_primitive;

typedef struct orc_texture {
    const void* data;
    uint32_t width, height, format, row_pitch; /* format: 0 RGBA8, 1 RGB32F */
} orc_texture;

typedef struct orc_scene {
    const orc_draw* draws;
    uint32_t draw_count;
    const float* transforms; /* 16 floats per node, column-major */
    const orc_primitive* primitives;
    const orc_material* materials;
    const orc_texture* textures;
    uint32_t texture_count;
} orc_scene;

/* Pyramid: mip k is max(1,w0>>k) x max(1,h0>>k) floats, packed. */
typedef struct orc_pyramid {
    float* data;
    uint32_t width, height, levels;
    /* the depth buffer it reduces (0: unknown; the fine occlusion test then
     * stays off) */
    uint32_t view_width, view_height;
} orc_pyramid;

enum {
    ORC_CULL_FRUSTUM = 1u << 0,
    ORC_CULL_OCCLUSION = 1u << 1,
    ORC_CULL_TWO_PASS = 1u << 2,
    ORC_CULL_CONE = 1u << 3,
    ORC_RESOLVE_FLAT = 1u << 4,
    ORC_RESOLVE_TEXTURED = 1u << 5,
    ORC_BUILD_PYRAMID = 1u << 6,
    ORC_CULL_OCCLUSION_FINE = 1u << 7
};

void orc_set_threads(int n);
int orc_get_threads(void);

uint32_t orc_pyramid_levels(uint32_t w, uint32_t h);
uint64_t orc_pyramid_floats(uint32_t w, uint32_t h);

/* Task shader for a candidate list (NULL = all draws).  pass 1 uses
 * prevOcclusionViewProjection, pass 2 occlusionViewProjection.
 * Survivors come out in ascending draw order.  rejected receives the draws
 * that passed the frustum test but failed the occlusion test. */
void orc_cull(const orc_scene* s, const orc_camera* cam, const orc_pyramid* pyr,
              uint32_t flags, uint32_t pass, const uint32_t* cand, uint32_t ncand,
              uint32_t* survivors, uint32_t* nsurv, uint32_t* rejected, uint32_t* nrej);

/* Mesh shader + fixed-function raster + fragment shader for a draw list. */
void orc_raster(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h,
                const uint32_t* draws, uint32_t ndraws, uint64_t* depth_id);

/* HiZ reduce chain (hiz_reduce.comp.glsl + application.cpp:951-1003). */
void orc_hiz(const uint64_t* depth_id, uint32_t w, uint32_t h, float* pyramid);

/* visbuffer_resolve.comp.glsl (flat) or the textured extension. */
void orc_resolve(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h,
                 const uint64_t* depth_id, uint32_t textured, uint32_t* ids, uint32_t* rgba);

/* Motion vectors of the visible fragments (visbuffer.frag.glsl:38): two
 * binary16 per pixel, x in the low half, 0 where nothing was drawn. */
void orc_motion(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h, const uint64_t* depth_id,
                uint32_t* motion);
/* binary32 -> binary16, round to nearest even (the conversion of the motion
 * attachment's stores). */
uint16_t orc_half_rn(float v);

/* A whole frame with the same pass structure as vkgv_frame. */
void orc_frame(const orc_scene* s, const orc_camera* cam, uint32_t w, uint32_t h,
               const orc_pyramid* prev, uint32_t flags, uint64_t* depth_id,
               uint32_t* ids, uint32_t* rgba, float* pyramid_out,
               uint32_t* survivors, uint32_t* nsurv);

/* Adjoint reference in float64 (the differentiable textured resolve, an
 * addition with no reference implementation).  Parameters are doubles so
 * that finite differences see the perturbation exactly.  For the visibility
 * ids of each pixel (0xFFFFFFFF = empty; draw index = meshlet index, identity
 * node transform):
 *   rgb = interp(colour) * albedo * bilinearREPEAT(texture, transformUv(interp(uv)))
 *   L   = scale * sum (rgb - target)^2
 * with perspective-correct barycentrics at the pixel centre's fp32 NDC
 * ((px + 0.5) / w * 2 - 1 in float, the point the GPU evaluates).
 * Returns L; writes rgb (if non-NULL) and ACCUMULATES the gradients into
 * gpos / gcol / gtex (each may be NULL). */
typedef struct orc_diff_scene {
    const orc_meshlet* meshlets;
    const uint32_t* vertex_indices;
    const uint8_t* tri_indices;
    const double* positions; /* 3 per vertex */
    const double* colors;    /* 3 per vertex */
    const double* uvs;       /* 2 per vertex */
    const double* texture;   /* 3 per texel */
    uint32_t tex_w, tex_h;
    double albedo[3], uv_offset[2], uv_scale[2], uv_rotation;
} orc_diff_scene;

double orc_diff_f64(const orc_diff_scene* s, const float vp[16], uint32_t w, uint32_t h, const uint32_t* ids,
                    const float* target, double scale, double* rgb, double* gpos, double* gcol, double* gtex,
                    int32_t* cells);
/* orc_diff_f64 with each covered pixel's bilinear cell held at freeze[2p],
 * freeze[2p+1] (NULL: none held); see oracle.c.  margin (if non-NULL)
 * receives, per pixel, the distance in texels from the sample to the nearest
 * texel-centre line (-1 for an empty pixel). */
double orc_diff_f64_frozen(const orc_diff_scene* s, const float vp[16], uint32_t w, uint32_t h, const uint32_t* ids,
                           const float* target, double scale, double* rgb, double* gpos, double* gcol, double* gtex,
                           int32_t* cells, const int32_t* freeze, double* margin);
/* cells (if non-NULL) receives, per pixel, the unwrapped bilinear cell
 * (floor(u*W - 0.5), floor(v*H - 0.5)), or INT32_MIN twice for an empty
 * pixel.  Bilinear filtering is only piecewise smooth: its derivative jumps
 * where a sample crosses a texel centre, so a finite difference in the
 * positions is a valid check of the analytic gradient only while no pixel's
 * cell changes across the stencil. */

/* ------------------------------------------------------------ world.c */
/* Node tree, animations and the per-frame transform / draw lists
 * (world.cpp:187-345, assets.hpp:51-113); the same layouts as the library's
 * vkgv_world_desc. */
typedef struct orc_node {
    float translation[3], rotation[4], scale[3]; /* rotation x, y, z, w */
    uint32_t mesh_index, first_child, child_count;
} orc_node; /* 52 B */

enum { ORC_PATH_TRANSLATION = 1, ORC_PATH_ROTATION = 2, ORC_PATH_SCALE = 3, ORC_PATH_WEIGHTS = 4 };
enum { ORC_INTERP_LINEAR = 0, ORC_INTERP_STEP = 1, ORC_INTERP_CUBICSPLINE = 2 };

typedef struct orc_anim_sampler {
    const float* input;
    const float* output;
    uint32_t input_count, output_count, interpolation, components;
} orc_anim_sampler;

typedef struct orc_anim_channel {
    uint32_t sampler, node, path, pad_;
} orc_anim_channel;

typedef struct orc_world {
    const orc_node* nodes;
    uint32_t node_count, child_count;
    const uint32_t* children;
    const uint32_t* roots;
    uint32_t root_count, mesh_count;
    const uint32_t* mesh_offsets;
    const uint32_t* mesh_primitives;
    const uint32_t* primitive_meshlet_counts;
    uint32_t primitive_count, sampler_count;
    const orc_anim_sampler* samplers;
    const orc_anim_channel* channels;
    uint32_t channel_count, pad_;
} orc_world;

/* World::updateTransformBuffer at animation_time: one column-major mat4 per
 * node with a mesh, in depth-first order.  Returns the count (-1 for a path
 * deeper than 64 nodes); writes at most `capacity` matrices. */
int64_t orc_world_transforms(const orc_world* w, float animation_time, float* transforms, uint32_t capacity);
/* World::rebuildDrawBuffer: MeshletDraw {primitive, meshlet, transform} as
 * three words each.  Returns the count (-1 as above). */
int64_t orc_world_draws(const orc_world* w, uint32_t* draws, uint64_t capacity);
/* The pinned pieces, exported for the CPU tests. */
void orc_anim_sample(const orc_anim_sampler* s, float time, uint32_t path, float out[4]);
void orc_slerp(const float a[4], const float b[4], float t, float out[4]);
void orc_trs_matrix(const float t[3], const float q[4], const float s[3], float m[16]);
float orc_sin_series(float x);
float orc_asin_series(float z);

/* ---------------------------------------------------------- texture.c */
/* BC1-BC5 blocks (format 1..5, row-major blocks of 8 or 16 bytes) into
 * RGBA8 texels (R in the low byte). */
void orc_decode_bc(uint32_t format, const uint8_t* blocks, uint32_t w, uint32_t h, uint32_t* rgba);
/* BC6H blocks -> binary16 bits, R, G, B per texel (is_signed: SF16). */
void orc_decode_bc6h(const uint8_t* blocks, uint32_t w, uint32_t h, int is_signed, uint16_t* rgb);
/* JPEG pixels from dequantized natural-order coefficient blocks: one
 * component's IDCT into an 8-bit plane (blocks_w * 8 wide), then the
 * upsampled colour conversion of 1 or 3 planes into RGBA8. */
void orc_jpeg_idct(const int16_t* coef, uint32_t blocks_w, uint32_t blocks_h, uint8_t* plane);
void orc_jpeg_color(const uint8_t* p0, const uint8_t* p1, const uint8_t* p2, const uint32_t pitch[3],
                    const uint32_t rx[3], const uint32_t ry[3], uint32_t w, uint32_t h, uint32_t components,
                    uint32_t rgb, uint32_t* out);

/* Single-fragment helpers exported for the known-answer tests. */
float orc_from_linear(float c);
float orc_to_linear(float c);
uint32_t orc_unorm8(float c);
/* Rasterises one clip-space triangle with a given id (KAT entry point). */
void orc_raster_triangle(const float v0[4], const float v1[4], const float v2[4],
                         uint32_t id, uint32_t w, uint32_t h, uint64_t* depth_id);
/* Min-reduction sample of a single-level image (KAT entry point). */
float orc_min_sample(const float* img, uint32_t w, uint32_t h, float u, float v);
int orc_frustum_visible(const float center[3], const float extents[3], const float planes[24]);

#ifdef __cplusplus
}
#endif
#endif
