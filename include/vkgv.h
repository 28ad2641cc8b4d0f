/*
 * vkgv.h — C ABI of the GB300 meshlet visibility-buffer path.
 *
 * This library replaces the Vulkan draw path of one headless vk_gltf_viewer
 * frame: task-shader meshlet culling, mesh-shader + fixed-function
 * visibility-buffer rasterisation, the HiZ min-pyramid reduction and the
 * visibility-buffer resolve.  The scene is consumed in the renderer's own
 * buffer layout (shaders/mesh_common.h.glsl:20-126,
 * shaders/visbuffer/visbuffer.h.glsl:20-56), with every buffer device address
 * being a CUDA device pointer instead of a VkDeviceAddress.
 *
 * Conventions
 *   - Every entry point returns an int status (VKGV_OK ...).  No C++
 *     exception crosses this boundary.  vkgv_last_error() explains the last
 *     non-OK status of a context.
 *   - The caller owns the scene, the cameras and every per-view output.  The
 *     context owns scratch (survivor lists, triangle bins, counters).
 *   - Calls are ordered on the CUDA stream passed in (a cudaStream_t given as
 *     void*; NULL is the legacy default stream).  A context is used by one
 *     host thread at a time, as the reference records its frame from one
 *     thread (src/vk_gltf_viewer/application.cpp:604-1280).
 *   - Device pointers are passed as uint64_t device addresses, mirroring the
 *     reference's buffer_reference push constants.
 */
#ifndef VKGV_H
#define VKGV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum vkgv_status {
    VKGV_OK = 0,
    VKGV_INVALID_ARG = 1,    /* null pointer, zero-size view, bad flag mix  */
    VKGV_OUT_OF_MEMORY = 2,  /* scratch allocation failed                   */
    VKGV_LIMIT_EXCEEDED = 3, /* draw count >= 2^25, view > 8192 px, ...     */
    VKGV_TIMEOUT = 4,        /* a bounded device wait ran out               */
    VKGV_CUDA_ERROR = 5,     /* a CUDA runtime call failed                  */
    VKGV_DEVICE_FAULT = 6    /* the device status word recorded a violation */
};

/* ------------------------------------------------------------- constants */
/* shaders/mesh_common.h.glsl:36-38 */
#define VKGV_MAX_VERTICES 64u
#define VKGV_MAX_PRIMITIVES 126u
#define VKGV_MAX_MESHLETS 102u
/* src/vk_gltf_viewer/assets.cpp:324 — the builder's triangle limit */
#define VKGV_BUILDER_MAX_TRIANGLES 124u
/* shaders/visbuffer/visbuffer.h.glsl:15-16, 67 */
#define VKGV_TRIANGLE_BITS 7u
#define VKGV_DRAW_INDEX_BITS 25u
#define VKGV_VISBUFFER_CLEAR 0xFFFFFFFFu
/* shaders/resource_table.h.glsl:23 */
#define VKGV_INVALID_HANDLE 0xFFFFFFFFu
/* largest view edge; keeps 28.8 fixed-point coordinates inside int32 */
#define VKGV_MAX_VIEW_DIM 8192u

/* ---------------------------------------------------- scene layout (A7) */
/* Byte-exact mirrors of the GLSL scalar-layout structs. */

/* glsl::Meshlet, shaders/mesh_common.h.glsl:49-58 — 36 bytes */
typedef struct vkgv_meshlet {
    uint32_t vertex_offset;   /* first entry in the vertex-index stream   */
    uint32_t triangle_offset; /* first byte in the triangle-index stream  */
    uint8_t vertex_count;
    uint8_t triangle_count;
    uint8_t _pad[2];
    float aabb_extents[3];
    float aabb_center[3];
} vkgv_meshlet;

/* glsl::Vertex, shaders/mesh_common.h.glsl:60-71 — 24 bytes */
typedef struct vkgv_vertex {
    float position[3];
    uint8_t color[4];   /* unpacked as color / 255 (mesh_common.h.glsl:74-76) */
    uint8_t normal[3];  /* unpacked as normal / 127 - 1 (mesh_common.h.glsl:78-80) */
    uint8_t _pad;
    uint16_t uv[2];     /* IEEE binary16 */
} vkgv_vertex;

/* glsl::MeshletDraw, shaders/mesh_common.h.glsl:96-100 — 12 bytes */
typedef struct vkgv_meshlet_draw {
    uint32_t primitive_index;
    uint32_t meshlet_index;
    uint32_t transform_index;
} vkgv_meshlet_draw;

/* glsl::Primitive, shaders/mesh_common.h.glsl:102-113 — 64 bytes, align 8 */
typedef struct vkgv_primitive {
    uint64_t vertex_index_buffer;    /* uint32 per meshlet vertex            */
    uint64_t primitive_index_buffer; /* uint8 triplets, meshlet-local        */
    uint64_t vertex_buffer;          /* vkgv_vertex                          */
    uint64_t meshlet_buffer;         /* vkgv_meshlet                         */
    float aabb_extents[3];
    float aabb_center[3];
    uint32_t meshlet_count;
    uint32_t material_index;
} vkgv_primitive;

/* glsl::Material, shaders/mesh_common.h.glsl:115-126 — 48 bytes */
typedef struct vkgv_material {
    float albedo_factor[4];
    uint32_t albedo_index; /* index into the scene's texture table, or VKGV_INVALID_HANDLE */
    float uv_offset[2];
    float uv_scale[2];
    float uv_rotation;
    float alpha_cutoff;
    uint32_t double_sided;
} vkgv_material;

/* glsl::Camera, shaders/mesh_common.h.glsl:20-27 — 352 bytes.
 * Matrices are column-major (m[column*4 + row]). */
typedef struct vkgv_camera {
    float prev_view_projection[16];
    float prev_occlusion_view_projection[16];
    float view_projection[16];
    float occlusion_view_projection[16];
    float frustum[6][4];
} vkgv_camera;

/* Texture descriptor: the bindless sampled-image table entry that
 * Material.albedoIndex names (shaders/resource_table.h.glsl:11). */
enum vkgv_texture_format {
    VKGV_TEXTURE_RGBA8 = 0,  /* 4 x uint8, sampled as UNORM then toLinear() */
    VKGV_TEXTURE_RGB32F = 1  /* 3 x float, linear                            */
};
typedef struct vkgv_texture {
    uint64_t data;       /* device address of texel (0,0)            */
    uint32_t width;
    uint32_t height;
    uint32_t format;     /* vkgv_texture_format                      */
    uint32_t row_pitch;  /* texels between rows (>= width)           */
} vkgv_texture;

/* HiZ pyramid: one R32_SFLOAT image with a full mip chain
 * (src/vk_gltf_viewer/application.cpp:472-529).  Mip 0 is (W>>1) x (H>>1);
 * mip k is max(1, (W>>1)>>k) x max(1, (H>>1)>>k); the mips are packed back
 * to back starting at `data`.  levels = floor(log2(max(W, H))). */
typedef struct vkgv_pyramid {
    uint64_t data;
    uint32_t width;   /* mip-0 width  = W >> 1 */
    uint32_t height;  /* mip-0 height = H >> 1 */
    uint32_t levels;  /* 0 = no pyramid */
    uint32_t _pad;
} vkgv_pyramid;

/* The scene half of glsl::VisbufferPushConstants
 * (shaders/visbuffer/visbuffer.h.glsl:37-47) plus the texture table. */
typedef struct vkgv_scene {
    uint64_t draw_buffer;        /* vkgv_meshlet_draw[meshlet_draw_count] */
    uint64_t transform_buffer;   /* float[16] per node, column-major      */
    uint64_t primitive_buffer;   /* vkgv_primitive[]                      */
    uint64_t material_buffer;    /* vkgv_material[]                       */
    uint64_t texture_table;      /* vkgv_texture[texture_count] or 0      */
    uint32_t meshlet_draw_count;
    uint32_t texture_count;
    /* Optional normal cones for VKGV_CULL_CONE: a device array of one
     * device address per primitive, each pointing at that primitive's
     * vkgv_meshlet_cone[meshlet_count] (0 = no cones for it). */
    uint64_t cone_table;
    uint32_t primitive_count;    /* entries of cone_table                 */
    /* Nodes in transform_buffer, or 0.  When given, a frame evaluates each
     * node's determinant (the winding sign of visbuffer.mesh.glsl:71) once
     * instead of once per meshlet draw; every transform_index must be below it. */
    uint32_t transform_count;
} vkgv_scene;

/* Normal cone of one meshlet in object space (an addition: glsl::Meshlet
 * has no cone, mesh_common.h.glsl:49-58, and the reference builds meshlets
 * with coneWeight 0, assets.cpp:323).  Every triangle normal n satisfies
 * dot(n, axis) >= cutoff and every vertex lies in the sphere (center,
 * radius).  cutoff <= 0 means the meshlet is never cone-culled.  32 bytes. */
typedef struct vkgv_meshlet_cone {
    float center[3];
    float radius;
    float axis[3];
    float cutoff;
} vkgv_meshlet_cone;

/* One headless view: the camera half of the push constants plus the
 * per-view images of the visbuffer, resolve and HiZ passes. */
typedef struct vkgv_view {
    uint64_t camera_buffer;      /* device address of one vkgv_camera       */
    uint32_t width;
    uint32_t height;
    vkgv_pyramid prev_pyramid;   /* read by the occlusion test; levels 0 = none */
    vkgv_pyramid pyramid;        /* written from this frame's depth          */
    uint64_t depth_id;           /* uint64[W*H]: (depth bits << 32) | (id + 1); 0 = clear */
    uint64_t visbuffer;          /* uint32[W*H] visbuffer IDs, or 0          */
    uint64_t color;              /* uint32[W*H] RGBA8 (R in the low byte), or 0 */
    uint64_t survivors;          /* uint32[survivor_capacity] drawn draw indices, or 0 */
    uint64_t survivor_count;     /* uint32 counter, or 0                     */
    uint32_t survivor_capacity;
    uint32_t _pad;
    /* uint32[W*H] motion vectors as two IEEE binary16 (x in the low half),
     * the visibility pass's second attachment (R16G16_SFLOAT,
     * application.cpp:250-270), written with VKGV_WRITE_MOTION, or 0 */
    uint64_t motion;
} vkgv_view;

/* ------------------------------------------------------------ frame flags */
enum vkgv_frame_flags {
    VKGV_CULL_FRUSTUM = 1u << 0,        /* isAabbInFrustum (culling.h.glsl:8-19)     */
    VKGV_CULL_OCCLUSION = 1u << 1,      /* HiZ test vs prev_pyramid (task.glsl:54-65) */
    VKGV_CULL_TWO_PASS = 1u << 2,       /* re-test pass-1 occlusion rejects vs this frame's pyramid */
    VKGV_CULL_CONE = 1u << 3,           /* conservative meshlet normal-cone test     */
    VKGV_RESOLVE_FLAT = 1u << 4,        /* visbuffer_resolve.comp.glsl               */
    VKGV_RESOLVE_TEXTURED = 1u << 5,    /* barycentrics + texture resolve            */
    VKGV_BUILD_PYRAMID = 1u << 6,       /* HiZ reduce chain into view.pyramid        */
    VKGV_WRITE_IDS = 1u << 7,           /* write the uint32 visbuffer image          */
    VKGV_SKIP_CLEAR = 1u << 8,          /* depth_id already cleared by the caller    */
    VKGV_WRITE_MOTION = 1u << 9,        /* motion vectors of the visible fragments (visbuffer.frag.glsl:38) */
    /* An addition to VKGV_CULL_OCCLUSION (no counterpart in the reference):
     * a draw that passes the HiZ test of visbuffer.task.glsl:54-65 is tested
     * again against every pyramid texel under its projected box, at the
     * finest exactly-halved level where that is at most 4 x 4 texels, and is
     * rejected when all of them hold a depth >= the box's nearest depth (the
     * reference's own comparison, on a finer footprint). */
    VKGV_CULL_OCCLUSION_FINE = 1u << 10,
    /* The reference frame: application.cpp:764-1003. */
    VKGV_FRAME_REFERENCE = (1u << 0) | (1u << 1) | (1u << 4) | (1u << 6) | (1u << 7)
};

/* --------------------------------------------------------------- context */
typedef struct vkgv_ctx vkgv_ctx;
typedef struct vkgv_graph vkgv_graph;

typedef struct vkgv_config {
    int32_t device;                  /* CUDA device ordinal                       */
    uint32_t bin_size;               /* raster bin edge in pixels: 8/16/32, 0 = default */
    uint32_t meshlets_per_cta;       /* meshlets per raster CTA: 1/2/4, 0 = default */
    uint32_t big_triangle_capacity;  /* binned-triangle queue entries, 0 = default */
    uint32_t spin_limit;             /* bounded device waits, 0 = default         */
    uint32_t _reserved[3];
} vkgv_config;

/* Replaces Application's device/pass initialisation
 * (src/vk_gltf_viewer/application.cpp:181-576). */
int vkgv_create(const vkgv_config* config, vkgv_ctx** out_ctx);
int vkgv_destroy(vkgv_ctx* ctx);
/* Human-readable reason of the last non-OK status on ctx (never NULL). */
const char* vkgv_last_error(const vkgv_ctx* ctx);
/* Reads and clears the device status word (first recorded violation). */
int vkgv_device_status(vkgv_ctx* ctx, uint32_t* out_code, uint32_t* out_detail);

/* One frame for `view_count` views: clear, cull (1 or 2 passes), raster,
 * pyramid, resolve as selected by `flags`.  Replaces the command recording
 * of Application::run (src/vk_gltf_viewer/application.cpp:764-1003).
 * view_count > 1 runs the batched path (all views in each launch). */
int vkgv_frame(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* views,
               uint32_t view_count, uint32_t flags, void* stream);

/* Stage entry points (each replaces one recorded pass). */
/* Clears depth_id to 0 and resets the survivor counter
 * (attachment clears, application.cpp:772-808). */
int vkgv_clear(vkgv_ctx* ctx, const vkgv_view* view, void* stream);
/* Task shader (shaders/visbuffer/visbuffer.task.glsl:25-76): appends the
 * surviving draw indices to view->survivors.  pass 1 tests against
 * view->prev_pyramid with prevOcclusionViewProjection; pass 2 re-tests the
 * pass-1 occlusion rejects against view->pyramid with
 * occlusionViewProjection (only the occlusion test: the rejects already
 * passed the frustum and cone tests of pass 1, whose camera fields
 * (frustum, view_projection) must not change in between). */
int vkgv_cull(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view,
              uint32_t flags, uint32_t pass, void* stream);
/* No counterpart in the reference.  vkgv_cull for callers that cannot
 * allocate device memory (a frame loop under global-mode stream capture, or
 * a plugin whose host owns every allocation): no context, no cudaMalloc.
 * Its scratch (view table, counters, status word, pass-1 reject list) is one
 * file-scope device array of about 1 MiB that every GPU loading the library
 * keeps until exit.  Scenes above 262,144 meshlet draws return
 * VKGV_LIMIT_EXCEEDED.  view->survivors and view->survivor_count are
 * required.  All calls share the array and leave its contents behind (pass 2
 * re-tests the rejects of the preceding pass-1 call); calls that overlap on
 * the GPU race.  The first call on a device looks up the array's device
 * address, so make it before any stream capture; the address is kept for the
 * lifetime of the device's primary context (not valid across a
 * cudaDeviceReset).  Device-side faults (an out-of-range meshlet index, a
 * full survivor list) are recorded in the array's status words, cleared by
 * each pass-1 call: read them with vkgv_cull_static_status. */
int vkgv_cull_static(const vkgv_scene* scene, const vkgv_view* view, uint32_t flags,
                     uint32_t pass, void* stream);
/* No counterpart in the reference.  Reads the status words that
 * vkgv_cull_static calls on the current device left since the last pass-1
 * call (code 0 = none; otherwise the first recorded fault, as
 * vkgv_device_status reports it) and clears them.  Ordered after the work on
 * `stream`, which it synchronises; allocates nothing. */
int vkgv_cull_static_status(void* stream, uint32_t* out_code, uint32_t* out_detail);
/* Mesh shader + raster + fragment shader
 * (shaders/visbuffer/visbuffer.mesh.glsl:30-104, visbuffer.frag.glsl:28-39):
 * rasterises draw_list[first .. *draw_count) into view->depth_id with a
 * 64-bit max, the order-independent equivalent of the GREATER_OR_EQUAL
 * depth test (application.cpp:333).  draw_list/draw_count are device
 * addresses; pass 0 for both to use view->survivors. */
int vkgv_raster(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view,
                uint64_t draw_list, uint64_t draw_count, uint32_t first, void* stream);
/* HiZ reduce chain (shaders/hiz_reduce.comp.glsl, application.cpp:951-1003):
 * view->depth_id -> view->pyramid. */
int vkgv_hiz_reduce(vkgv_ctx* ctx, const vkgv_view* view, void* stream);
/* Resolve (shaders/visbuffer/visbuffer_resolve.comp.glsl:17-41): writes
 * view->color (and view->visbuffer with VKGV_WRITE_IDS).  flags selects
 * VKGV_RESOLVE_FLAT or VKGV_RESOLVE_TEXTURED; VKGV_WRITE_MOTION also writes
 * view->motion, the visible fragments' motion vectors
 * (visbuffer.frag.glsl:38), from the camera's prev_view_projection. */
int vkgv_resolve(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view,
                 uint32_t flags, void* stream);

/* GPU stage zones, the analogue of the reference's GPU profiler zones
 * (TracyVkZone at application.cpp:765, 919, 952).  While enabled, every
 * vkgv_frame outside graph capture records a CUDA event at each stage
 * boundary; vkgv_stage_times waits for the last such frame and returns the
 * milliseconds of each stage in this order: clear, cull pass 1, meshlet
 * raster pass 1, binned raster pass 1, pyramid pass 1, cull pass 2,
 * meshlet raster pass 2, binned raster pass 2, pyramid, resolve, finalise
 * (VKGV_STAGE_COUNT entries; 0 for stages that did not run). */
#define VKGV_STAGE_COUNT 11u
int vkgv_set_profiling(vkgv_ctx* ctx, int32_t enable);
int vkgv_stage_times(vkgv_ctx* ctx, float* out_ms, uint32_t count);

/* Pyramid geometry for a W x H view: levels and total float count. */
int vkgv_pyramid_layout(uint32_t width, uint32_t height, uint32_t* out_levels,
                        uint64_t* out_float_count);

/* Captures one vkgv_frame into a CUDA graph (the buffers named by scene and
 * views are baked in; camera contents may change between launches). */
int vkgv_graph_capture(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* views,
                       uint32_t view_count, uint32_t flags, vkgv_graph** out_graph);
int vkgv_graph_launch(vkgv_graph* graph, void* stream);
int vkgv_graph_destroy(vkgv_graph* graph);
/* Number of kernel launches one vkgv_graph_launch performs. */
int vkgv_graph_kernel_count(const vkgv_graph* graph, uint32_t* out_count);

/* ------------------------------------------------------------- autotuner */
/* An addition with no reference counterpart (the reference's mesh-shader
 * workgroup sizes are fixed at pipeline creation).  Sweeps raster bin size
 * {8, 16, 32} x meshlets per CTA {1, 2, 4}: for each candidate a context
 * built from `base` with those two fields captures this frame as a graph,
 * launches it once to warm up, then `launches` times between CUDA events on
 * a private stream.  The candidates render into the caller's views (every
 * candidate produces the same visibility; the parity tests cover each).
 * Writes up to entry_capacity entries (in sweep order) and the fastest
 * configuration into *best. */
typedef struct vkgv_tune_entry {
    uint32_t bin_size;
    uint32_t meshlets_per_cta;
    float ms_per_launch;
    uint32_t _pad;
} vkgv_tune_entry;

int vkgv_autotune(const vkgv_config* base, const vkgv_scene* scene, const vkgv_view* views, uint32_t view_count,
                  uint32_t flags, uint32_t launches, vkgv_tune_entry* entries, uint32_t entry_capacity,
                  uint32_t* out_entry_count, vkgv_config* best);

/* ------------------------------------------------ adjoint of the resolve */
/* An addition with no reference implementation: a differentiable form of
 * the textured resolve (the commented-out visbuffer.frag.glsl:29-34) over
 * fp32 parameters.  Shading is linear RGB
 *     rgb = interp(colour) * albedo * tex(transformUv(interp(uv)))
 * with perspective-correct barycentrics of the visible triangle and a
 * bilinear REPEAT fp32 RGB texture.  Visibility comes from the regular cull
 * and raster kernels (identity node transform) and is recomputed in the
 * backward pass instead of being stored. */
typedef struct vkgv_diff_scene {
    uint64_t meshlet_buffer;          /* vkgv_meshlet[meshlet_count]        */
    uint64_t vertex_index_buffer;     /* uint32 meshlet vertex indices      */
    uint64_t primitive_index_buffer;  /* uint8 meshlet-local triplets       */
    uint64_t positions;               /* float[3 * vertex_count]            */
    uint64_t colors;                  /* float[3 * vertex_count], linear    */
    uint64_t uvs;                     /* float[2 * vertex_count]            */
    uint64_t texture;                 /* float[3 * tex_width * tex_height]  */
    uint32_t meshlet_count;
    uint32_t vertex_count;
    uint32_t tex_width;
    uint32_t tex_height;
    float albedo[3];
    float uv_offset[2];
    float uv_scale[2];
    float uv_rotation;
    uint32_t double_sided;
    /* Meshlet normal-cone culling of the visibility passes (cones rebuilt
     * from the current positions; the visibility is unchanged):
     * 0 = automatic (on for large batches), 1 = always, 2 = never. */
    uint32_t cone_mode;
} vkgv_diff_scene;

typedef struct vkgv_diff_view {
    uint64_t camera_buffer;  /* device vkgv_camera                         */
    uint32_t width, height;
    uint64_t depth_id;       /* uint64[W*H] visibility scratch, 16-byte aligned */
    uint64_t rgb;            /* float[3*W*H] shaded output, or 0           */
    uint64_t target;         /* float[3*W*H] MSE target (backward), or 0   */
    uint64_t grad_rgb;       /* float[3*W*H] dL/drgb (backward, used when target is 0) */
} vkgv_diff_view;

/* Renders every view's shaded linear RGB into view.rgb. */
int vkgv_diff_forward(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views,
                      uint32_t view_count, void* stream);
/* Backward pass.  With view.target: L = scale * sum over views, pixels and
 * channels of (rgb - target)^2 (empty pixels contribute target^2), which is
 * accumulated into *loss.  Without a target, view.grad_rgb gives dL/drgb.
 * Accumulates dL/dpositions, dL/dcolors and dL/dtexels into the three
 * gradient arrays (fp32 atomics; zero them first); any of them may be 0. */
int vkgv_diff_backward(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views,
                       uint32_t view_count, float scale, uint64_t loss, uint64_t grad_positions,
                       uint64_t grad_colors, uint64_t grad_texture, void* stream);

/* Passes recorded by vkgv_diff_graph_capture, in this order. */
enum {
    VKGV_DIFF_ZERO_GRADS = 1, /* memset loss and the gradient arrays to 0    */
    VKGV_DIFF_FORWARD = 2,    /* visibility + shading into view.rgb          */
    VKGV_DIFF_BACKWARD = 4    /* visibility recomputed + gradients           */
};
/* Captures the selected passes over these views into one CUDA graph (a
 * training step: zero, forward, backward), launched with vkgv_graph_launch.
 * Pointers, sizes, scale and view count are baked in; parameter, camera and
 * target contents may change between launches. */
int vkgv_diff_graph_capture(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views,
                            uint32_t view_count, uint32_t passes, float scale, uint64_t loss,
                            uint64_t grad_positions, uint64_t grad_colors, uint64_t grad_texture,
                            vkgv_graph** out_graph);

/* ------------------------------------------------------------------ world */
/* The node tree, its animations and the per-frame buffers built from it
 * (src/vk_gltf_viewer/world.cpp:187-345, include/vk_gltf_viewer/assets.hpp:51-113):
 * World::updateTransformBuffer becomes vkgv_world_update_transforms and
 * World::rebuildDrawBuffer vkgv_world_build_draws, both on the device.  The
 * tree is walked depth-first from the roots as World::iterateNode does; every
 * visit of a node with a mesh takes the next transform index, and its
 * primitives' meshlets append MeshletDraw records in that order. */

/* A glTF node after DecomposeNodeMatrices (fastgltf::TRS). */
typedef struct vkgv_node {
    float translation[3];
    float rotation[4];      /* quaternion x, y, z, w */
    float scale[3];
    uint32_t mesh_index;    /* VKGV_INVALID_HANDLE: no mesh */
    uint32_t first_child;   /* children at vkgv_world_desc.children[first_child, +child_count) */
    uint32_t child_count;
} vkgv_node; /* 52 B */

enum vkgv_anim_path {
    VKGV_PATH_TRANSLATION = 1,
    VKGV_PATH_ROTATION = 2,
    VKGV_PATH_SCALE = 3,
    VKGV_PATH_WEIGHTS = 4   /* accepted and ignored, as the reference does */
};

enum vkgv_anim_interpolation {
    VKGV_INTERP_LINEAR = 0,
    VKGV_INTERP_STEP = 1,
    VKGV_INTERP_CUBICSPLINE = 2
};

/* An animation sampler (assets.hpp:37-47): keyframe times and outputs, host
 * arrays copied to the device by vkgv_world_create. */
typedef struct vkgv_anim_sampler {
    const float* input;      /* input_count times, ascending */
    const float* output;     /* output_count * components floats */
    uint32_t input_count;
    uint32_t output_count;   /* input_count, or 3 * input_count for CUBICSPLINE */
    uint32_t interpolation;  /* vkgv_anim_interpolation */
    uint32_t components;     /* 3 (translation, scale), 4 (rotation), 1 (weights, unused) */
} vkgv_anim_sampler;

/* A channel; channels apply in array order (the reference's animation by
 * animation, channel by channel), a later one overriding an earlier one. */
typedef struct vkgv_anim_channel {
    uint32_t sampler;        /* index into vkgv_world_desc.samplers */
    uint32_t node;           /* VKGV_INVALID_HANDLE: no target */
    uint32_t path;           /* vkgv_anim_path */
    uint32_t _pad;
} vkgv_anim_channel;

/* Host arrays describing one world (World::addAsset's merged tables). */
typedef struct vkgv_world_desc {
    const vkgv_node* nodes;
    uint32_t node_count;
    uint32_t child_count;
    const uint32_t* children;
    const uint32_t* roots;              /* scenes[0].nodeIndices */
    uint32_t root_count;
    uint32_t mesh_count;
    const uint32_t* mesh_offsets;       /* mesh_count + 1 offsets into mesh_primitives */
    const uint32_t* mesh_primitives;    /* Mesh::primitiveIndices, concatenated */
    const uint32_t* primitive_meshlet_counts; /* PrimitiveBuffers::meshletCount */
    uint32_t primitive_count;
    uint32_t sampler_count;
    const vkgv_anim_sampler* samplers;
    const vkgv_anim_channel* channels;
    uint32_t channel_count;
    uint32_t _pad;
} vkgv_world_desc;

#define VKGV_MAX_NODE_DEPTH 64u

typedef struct vkgv_world vkgv_world;
/* Validates the tables, walks the tree once on the host (the draw and
 * transform order never changes afterwards, as world.cpp:236-238 assumes)
 * and uploads the plan and the keyframes.  A path deeper than
 * VKGV_MAX_NODE_DEPTH (or a cycle) is VKGV_LIMIT_EXCEEDED. */
int vkgv_world_create(vkgv_ctx* ctx, const vkgv_world_desc* desc, vkgv_world** out_world);
int vkgv_world_destroy(vkgv_world* world);
/* Transform slots (mesh-node visits) and MeshletDraw records of the world. */
int vkgv_world_info(const vkgv_world* world, uint32_t* out_transform_count, uint64_t* out_draw_count);
/* World::updateTransformBuffer at animationTime: samples every channel,
 * composes parent * T * R * S down the tree and writes one column-major
 * mat4 per transform slot into transform_buffer (device float[16 * T]). */
int vkgv_world_update_transforms(vkgv_ctx* ctx, vkgv_world* world, float animation_time,
                                 uint64_t transform_buffer, void* stream);
/* World::rebuildDrawBuffer: writes the MeshletDraw list on the device into
 * draw_buffer (16-byte aligned, capacity >= the draw count). */
int vkgv_world_build_draws(vkgv_ctx* ctx, vkgv_world* world, uint64_t draw_buffer, uint64_t capacity,
                           void* stream);

/* ------------------------------------------------------------ glTF import */
/* A glTF 2.0 asset (.glb, or .gltf with external or base64 data: buffers)
 * read into the renderer's layout, as src/vk_gltf_viewer/assets.cpp:288-552
 * and World::addAsset (world.cpp:9-80) do with fastgltf: POSITION (float or
 * KHR_mesh_quantization integers), indices (generated when absent), meshlets
 * of 64 vertices / 124 triangles, material index + 1 (0 = the default
 * material), baseColorFactor, alphaCutoff, doubleSided, node matrices
 * decomposed into TRS, the first scene's root nodes, and every animation's
 * samplers and channels.  COLOR_0 and TEXCOORD_0 are kept when present.
 * EXT_meshopt_compression buffer views are decoded (vkgv_meshopt_decode,
 * the views in parallel); fallback buffers are never read. */
typedef struct vkgv_gltf vkgv_gltf;

/* Also store baseColorTexture's texture index and its KHR_texture_transform
 * in the materials (the reference leaves albedoIndex invalid,
 * assets.cpp:510-514, and loads no images). */
#define VKGV_GLTF_TEXTURE_REFERENCES 1u
/* Also read every texture's encoded image (a file, a data URI or a
 * bufferView; the MSFT_texture_dds source when present) for
 * vkgv_gltf_get_texture_image. */
#define VKGV_GLTF_IMAGES 2u

enum vkgv_image_kind {
    VKGV_IMAGE_UNKNOWN = 0,
    VKGV_IMAGE_PNG = 1,
    VKGV_IMAGE_DDS = 2,
    VKGV_IMAGE_JPEG = 3,
    VKGV_IMAGE_KTX2 = 4
};

typedef struct vkgv_gltf_image {
    const uint8_t* data;   /* encoded bytes, owned by the asset (NULL: none) */
    uint64_t size;
    uint32_t kind;         /* vkgv_image_kind, from the magic bytes */
    uint32_t _pad;
} vkgv_gltf_image;

typedef struct vkgv_gltf_info {
    uint32_t primitive_count;
    uint32_t material_count;   /* glTF materials + 1 */
    uint32_t mesh_count;
    uint32_t node_count;
    uint32_t root_count;
    uint32_t sampler_count;
    uint32_t channel_count;
    uint32_t texture_count;
    uint32_t image_count;
    uint32_t _pad;
} vkgv_gltf_info;

typedef struct vkgv_gltf_primitive {
    struct vkgv_mesh* mesh;    /* meshletised streams, owned by the asset */
    uint32_t material_index;   /* glTF material + 1, 0 = default (assets.cpp:290-293) */
    uint32_t mesh_index;       /* the glTF mesh it belongs to */
    uint32_t meshlet_count;
    uint32_t _pad;
} vkgv_gltf_primitive;

/* On failure returns a status and writes a message into error (if given). */
int vkgv_gltf_load(const char* path, uint32_t flags, vkgv_gltf** out_asset, char* error,
                   uint32_t error_capacity);
int vkgv_gltf_get_info(const vkgv_gltf* asset, vkgv_gltf_info* out);
int vkgv_gltf_get_primitive(const vkgv_gltf* asset, uint32_t index, vkgv_gltf_primitive* out);
/* Copies material_count materials (index 0 = the glTF default). */
int vkgv_gltf_get_materials(const vkgv_gltf* asset, vkgv_material* out, uint32_t capacity);
/* The node tree, meshes and animations as a vkgv_world_desc whose arrays
 * live until vkgv_gltf_free. */
int vkgv_gltf_get_world(const vkgv_gltf* asset, vkgv_world_desc* out);
/* The encoded image of texture `texture` (loaded with VKGV_GLTF_IMAGES). */
int vkgv_gltf_get_texture_image(const vkgv_gltf* asset, uint32_t texture, vkgv_gltf_image* out);
void vkgv_gltf_free(vkgv_gltf* asset);

/* One EXT_meshopt_compression bufferView: `size` bytes of stream at src
 * decoded into count x stride bytes at dst (host memory), then filtered in
 * place.  Replaces the per-view body of MeshoptDecompressor::ExecuteRange
 * (src/vk_gltf_viewer/assets.cpp:111-166), which calls meshoptimizer's
 * meshopt_decodeVertexBuffer / meshopt_decodeIndexBuffer /
 * meshopt_decodeIndexSequence and meshopt_decodeFilterOct / Quat / Exp.
 * Strides: ATTRIBUTES a multiple of 4 up to 256 (OCTAHEDRAL 4 or 8,
 * QUATERNION 8); TRIANGLES and INDICES 2 or 4, TRIANGLES count a multiple
 * of 3; filters only with ATTRIBUTES.  VKGV_INVALID_ARG for anything else
 * and for a stream that does not decode to exactly its declared size (the
 * reference ignores that status, assets.cpp:146-147). */
typedef enum vkgv_meshopt_mode {
    VKGV_MESHOPT_ATTRIBUTES = 0,
    VKGV_MESHOPT_TRIANGLES = 1,
    VKGV_MESHOPT_INDICES = 2
} vkgv_meshopt_mode;

typedef enum vkgv_meshopt_filter {
    VKGV_MESHOPT_FILTER_NONE = 0,
    VKGV_MESHOPT_FILTER_OCTAHEDRAL = 1,
    VKGV_MESHOPT_FILTER_QUATERNION = 2,
    VKGV_MESHOPT_FILTER_EXPONENTIAL = 3
} vkgv_meshopt_filter;

int vkgv_meshopt_decode(void* dst, uint64_t count, uint64_t stride, const void* src, uint64_t size, int mode,
                        int filter);

/* -------------------------------------------------------- texture decode */
/* Base-colour images for the textured resolve.  The reference's image
 * loading is an empty task (src/vk_gltf_viewer/assets.cpp:467-471); these
 * decode the published formats: PNG on the host (own DEFLATE), and the
 * block-compressed formats of DDS files (MSFT_texture_dds) on the device. */
typedef struct vkgv_image vkgv_image;

/* PNG (all colour types and bit depths, Adam7, tRNS) -> RGBA8 on the host;
 * 16-bit samples keep their high byte.  On failure a message goes to
 * error (if given). */
int vkgv_image_decode_png(const void* data, uint64_t size, vkgv_image** out_image, char* error,
                          uint32_t error_capacity);
/* Size and RGBA8 pixels (row-major, R in the low byte) of a decoded image. */
int vkgv_image_get(const vkgv_image* image, uint32_t* width, uint32_t* height, const uint8_t** rgba);
void vkgv_image_free(vkgv_image* image);

enum vkgv_block_format {
    VKGV_BC1 = 1,   /* DXT1: RGB565 pair + 2-bit indices (1-bit alpha when c0 <= c1) */
    VKGV_BC2 = 2,   /* DXT3: explicit 4-bit alpha + BC1 colours                      */
    VKGV_BC3 = 3,   /* DXT5: interpolated alpha + BC1 colours                        */
    VKGV_BC4 = 4,   /* one interpolated channel (R)                                  */
    VKGV_BC5 = 5,   /* two interpolated channels (R, G)                              */
    VKGV_BC1_OPAQUE = 6, /* BC1 read as Vulkan's BC1_RGB formats: the three-colour
                          * mode's fourth entry is opaque black                      */
    VKGV_RGBA8 = 7, /* uncompressed RGBA8 texels (reported by vkgv_ktx2_parse only;
                     * not a vkgv_decode_bc format)                                 */
    VKGV_BC7 = 8,   /* BPTC UNORM: eight modes of 1-3 subsets, 16-byte blocks       */
    VKGV_BC6H_UF16 = 9,  /* BPTC float, unsigned: fourteen modes of 1-2 regions,
                          * binary16 RGB texels (vkgv_decode_bc6h)                  */
    VKGV_BC6H_SF16 = 10, /* BPTC float, signed                                      */
    /* uncompressed 32-bit DDS texels (reported by vkgv_dds_parse; decoded on
     * the host): B, G, R, A bytes; and R, G, B / B, G, R bytes with a fourth
     * byte that is not alpha (read as 255) */
    VKGV_BGRA8 = 11,
    VKGV_RGBX8 = 12,
    VKGV_BGRX8 = 13
};

typedef struct vkgv_dds_info {
    uint32_t width;
    uint32_t height;
    uint32_t mip_count;
    uint32_t format;         /* vkgv_block_format */
    uint32_t srgb;           /* DXGI *_UNORM_SRGB, or a KTX2 *_SRGB vkFormat */
    uint32_t supercompression; /* KTX2: 0 none, 2 Zstandard (data_offset / data_size
                                * then hold the compressed level; it decodes with
                                * vkgv_zstd_decompress to the format's texel size) */
    uint64_t data_offset;    /* byte offset of the top mip's blocks */
    uint64_t data_size;      /* bytes of the top mip */
} vkgv_dds_info;

/* Reads a DDS header (FourCC DXT1-5 / ATI1 / ATI2 / BC4U / BC5U, or DX10
 * with a BC1-BC5, BC6H (UF16 / SF16) or BC7 DXGI format), or an uncompressed
 * 32-bit one: DX10 R8G8B8A8 (28, 29), B8G8R8A8 (87, 91), B8G8R8X8 (88, 93),
 * or a DDPF_RGB pixel format with RGBA / BGRA byte masks (format VKGV_RGBA8,
 * VKGV_BGRA8, or VKGV_RGBX8 / VKGV_BGRX8 without DDPF_ALPHAPIXELS);
 * VKGV_INVALID_ARG for anything else. */
int vkgv_dds_parse(const void* data, uint64_t size, vkgv_dds_info* out);
/* Reads a KTX 2.0 header (the container of KHR_texture_basisu, which the
 * reference enables in fastgltf, assets.cpp:539, and links ktx_read for):
 * a 2D texture (one layer, one face), without supercompression or with
 * Zstandard supercompression (scheme 2), whose vkFormat is BC1-BC5 UNORM /
 * SRGB (131-139, 141), BC6H UFLOAT / SFLOAT (143, 144), BC7 UNORM / SRGB
 * (145, 146) or R8G8B8A8 UNORM / SRGB
 * (37, 43), into the same
 * fields as a DDS file (level 0; format VKGV_BC1_OPAQUE for BC1_RGB,
 * VKGV_RGBA8 for R8G8B8A8; `supercompression` set to 2 for a zstd level,
 * whose uncompressed length must be the format's texel size).  BasisU
 * (vkFormat 0, BasisLZ scheme 1), SNORM formats, cube maps, arrays and 3D
 * textures are VKGV_INVALID_ARG. */
int vkgv_ktx2_parse(const void* data, uint64_t size, vkgv_dds_info* out);
/* Zstandard (RFC 8878) decoder for KTX2 supercompression scheme 2 (libktx,
 * which the reference links as ktx_read, CMakeLists.txt:13, inflates these
 * with libzstd): decodes every frame of src (skippable frames skipped, no
 * dictionaries, content checksums verified) into dst.  *out_size receives
 * the decoded length.  VKGV_LIMIT_EXCEEDED when dst_capacity is too small,
 * VKGV_INVALID_ARG for a corrupt or truncated stream.  Host only. */
int vkgv_zstd_decompress(const void* src, uint64_t src_size, void* dst, uint64_t dst_capacity,
                         uint64_t* out_size);
/* XXH64 (seed 0) of data, the hash of the zstd content checksum. */
uint64_t vkgv_xxh64(const void* data, uint64_t size);
/* Decodes width x height texels of BC1-BC5 or BC7 blocks (device,
 * row-major blocks of 8 or 16 bytes, aligned to the block size) into RGBA8
 * (device uint32[width * height], 4-byte aligned). */
int vkgv_decode_bc(vkgv_ctx* ctx, uint32_t format, uint64_t blocks, uint32_t width, uint32_t height,
                   uint64_t rgba_out, void* stream);
/* Decodes width x height texels of BC6H blocks (format VKGV_BC6H_UF16 or
 * VKGV_BC6H_SF16; device, row-major 16-byte blocks, 16-byte aligned) into
 * float32 R, G, B per texel (device float[width * height * 3], 4-byte
 * aligned): the binary16 values of the format, exactly, for a linear
 * VKGV_TEXTURE_RGB32F texture.  Reserved modes decode to 0.  (The
 * reference enables MSFT_texture_dds, assets.cpp:540, whose DDS files may
 * hold BC6H.) */
int vkgv_decode_bc6h(vkgv_ctx* ctx, uint32_t format, uint64_t blocks, uint32_t width, uint32_t height,
                     uint64_t rgb_out, void* stream);

/* JPEG (the reference links wuffs for it, wuffs_implementation.cpp:1-5):
 * sequential or progressive DCT, Huffman, 8-bit; 1 component or 3 (YCbCr,
 * or RGB per an Adobe transform 0 / component ids 'R','G','B'); sampling
 * factors 1-4 with integral ratios; restart intervals; interleaved or
 * single-component scans.  Lossless, hierarchical and arithmetic-coded
 * files are refused.
 * The entropy decode runs on the host into dequantized coefficient planes;
 * vkgv_jpeg_to_rgba runs the IDCT, chroma upsampling (replication) and the
 * JFIF colour conversion on the device, in pinned fixed-point arithmetic. */
typedef struct vkgv_jpeg vkgv_jpeg;

typedef struct vkgv_jpeg_info {
    uint32_t width;
    uint32_t height;
    uint32_t components;     /* 1 or 3 */
    uint32_t rgb;            /* 3 components stored as R, G, B (no YCbCr conversion) */
    uint32_t hmax;           /* largest sampling factors */
    uint32_t vmax;
    uint32_t h[3];           /* sampling factors per component */
    uint32_t v[3];
    uint32_t blocks_w[3];    /* coefficient planes, in 8x8 blocks (MCU-padded) */
    uint32_t blocks_h[3];
} vkgv_jpeg_info;

int vkgv_jpeg_decode_coefficients(const void* data, uint64_t size, vkgv_jpeg** out_jpeg, char* error,
                                  uint32_t error_capacity);
int vkgv_jpeg_get_info(const vkgv_jpeg* jpeg, vkgv_jpeg_info* out);
/* Component c's blocks_w x blocks_h blocks in raster order, each 64 int16
 * coefficients in natural (row-major) order, already multiplied by the
 * quantisation step (clamped to int16). */
int vkgv_jpeg_get_coefficients(const vkgv_jpeg* jpeg, uint32_t component, const int16_t** out);
/* IDCT + upsampling + colour conversion into width x height RGBA8 (device
 * uint32[], 4-byte aligned; alpha 255); the coefficients are copied in
 * through the context's scratch, so the vkgv_jpeg may be freed on return. */
int vkgv_jpeg_to_rgba(vkgv_ctx* ctx, const vkgv_jpeg* jpeg, uint64_t rgba_out, void* stream);
void vkgv_jpeg_free(vkgv_jpeg* jpeg);

/* ---------------------------------------------- host scene producers (A15) */
/* Replace the glTF import + meshletiser (src/vk_gltf_viewer/assets.cpp:288-430)
 * for procedural scenes, and the camera update (src/vk_gltf_viewer/camera.cpp). */
typedef struct vkgv_mesh vkgv_mesh;

typedef struct vkgv_mesh_info {
    uint32_t vertex_count;
    uint32_t triangle_count;
    uint32_t meshlet_count;
    uint32_t vertex_index_count;     /* entries in the vertex-index stream   */
    uint32_t primitive_index_bytes;  /* bytes in the triangle-index stream   */
    float position_scale;            /* dequantisation scale a node matrix must apply
                                        (KHR_mesh_quantization); 1 when unquantised */
    const vkgv_vertex* vertices;
    const float* positions;          /* float3 per vertex (unquantised source) */
    const float* uvs;                /* float2 per vertex                      */
    const uint32_t* indices;         /* uint32 x 3 per triangle                */
    const vkgv_meshlet* meshlets;
    const uint32_t* vertex_indices;
    const uint8_t* primitive_indices;
    float aabb_extents[3];
    float aabb_center[3];
    const vkgv_meshlet_cone* cones;  /* one per meshlet                   */
} vkgv_mesh_info;

/* Icosahedron subdivided `level` times onto the unit sphere
 * (20 * 4^level triangles). */
vkgv_mesh* vkgv_mesh_icosphere(uint32_t level);
/* Torus (ring radius R, tube radius r) with seg_major x seg_minor quads,
 * displaced along the normal by seeded value noise of amplitude noise_amp.
 * quantize != 0 stores positions as KHR_mesh_quantization int16-normalised
 * values (dequantised into vkgv_vertex.position) and normals as int8. */
vkgv_mesh* vkgv_mesh_torus(float R, float r, uint32_t seg_major, uint32_t seg_minor,
                           float noise_amp, uint64_t seed, int32_t quantize);
/* Displaces an icosphere-like mesh along its normalised position by seeded
 * value noise (amplitude amp). */
int vkgv_mesh_displace(vkgv_mesh* mesh, float amp, uint64_t seed);
/* Mesh from caller arrays (positions float3, indices uint32 x 3). */
vkgv_mesh* vkgv_mesh_from_arrays(const float* positions, uint32_t vertex_count,
                                 const uint32_t* indices, uint32_t triangle_count);
/* Sets per-vertex RGBA8 colours and binary16 UVs from float arrays
 * (either may be NULL). */
int vkgv_mesh_set_attributes(vkgv_mesh* mesh, const float* rgba, const float* uv);
/* Greedy meshletiser with the reference limits (64 vertices / 124
 * triangles; assets.cpp:323-341); also computes each meshlet AABB
 * (assets.cpp:348-372). */
int vkgv_mesh_build_meshlets(vkgv_mesh* mesh, uint32_t max_vertices, uint32_t max_triangles);
int vkgv_mesh_get_info(const vkgv_mesh* mesh, vkgv_mesh_info* out);
void vkgv_mesh_free(vkgv_mesh* mesh);

/* Camera update (src/vk_gltf_viewer/camera.cpp:170-193): shifts the current
 * matrices into prev*, writes VP = reverseZ * perspectiveRH_ZO(y-flip) *
 * lookAtRH, copies it to occlusionViewProjection and extracts the six
 * frustum planes. */
int vkgv_camera_update(vkgv_camera* camera, const float eye[3], const float target[3],
                       const float up[3], float fovy_radians, float aspect,
                       float znear, float zfar);
/* Frustum planes of a view-projection (camera.cpp:70-84). */
int vkgv_frustum_planes(const float view_projection[16], float out_planes[24]);

/* Library version string. */
const char* vkgv_version(void);

#ifdef __cplusplus
}
#endif
#endif /* VKGV_H */
