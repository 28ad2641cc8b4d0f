// Kernel launchers shared between the translation units of libvkgv.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

namespace vkgv {

// Launches a frame kernel with programmatic stream serialisation (the
// kernel calls pdl_begin() before touching its predecessor's results).
template <typename... Params, typename... Args>
inline void launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                       Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

struct RasterLists {
    uint32_t pass;            // 1, 2, or 0 for an explicit list
    const uint32_t* list;     // explicit list (pass 0)
    const uint32_t* count;    // explicit count (pass 0), device
    uint32_t first;           // explicit start (pass 0)
    uint32_t deferred_slot;   // DeviceView::counters index of this raster's deferred list (4, 5, 6)
};

struct RasterConfig {
    uint32_t small_area;      // bbox pixel area rasterised inline by the lane
    uint32_t chunk;           // edge of the binned chunk in pixels (8, 16, 32, 64)
    uint32_t warps_per_cta;   // meshlets in flight per CTA
    uint32_t blocks_per_view;
};

// Zeroes the views' depth_id (unless max_pixels is 0) and, when counters is
// not null, the global and per-view counters.  Also evaluates, when
// transform_count > 0, determinant(M) of transforms[0, transform_count) into
// tdets and each view's view_projection * M into its DeviceView::mvps table
// (and prev_view_projection * M into DeviceView::prev_mvps where that is set);
// mvps is the tables' allocation, null to skip them.
void launch_clear(const DeviceView* views, uint32_t nviews, uint64_t max_pixels, uint32_t* counters,
                  uint32_t counter_words, uint32_t sm_count, cudaStream_t stream, const float* transforms = nullptr,
                  uint32_t transform_count = 0, float* tdets = nullptr, float* mvps = nullptr);
void launch_cull(const SceneArgs& S, const DeviceView* views, uint32_t nviews, uint32_t flags, uint32_t pass,
                 uint32_t* status, uint32_t sm_count, cudaStream_t stream);
// work: two counters that are zero between launches (each launch returns
// them to zero).
void launch_raster(const SceneArgs& S, const DeviceView* views, uint32_t nviews, const RasterLists& lists,
                   const RasterConfig& cfg, BigTri* big, uint32_t* big_count, uint32_t big_capacity,
                   uint32_t* work, uint32_t* status, uint32_t sm_count, cudaStream_t stream,
                   cudaEvent_t between = nullptr);
// Shared-memory floats the HiZ tail needs for a view: the texels of its
// levels above the tiled ones.
uint32_t hiz_tail_floats(uint32_t w, uint32_t h, uint32_t levels);
void launch_hiz(const DeviceView* views, uint32_t nviews, uint32_t tiles_x, uint32_t tiles_y, uint32_t tail,
                uint32_t* status, cudaStream_t stream);
void launch_resolve(const SceneArgs& S, const DeviceView* views, uint32_t nviews, uint32_t max_w, uint32_t max_h,
                    uint32_t flags, uint32_t* work, uint32_t sm_count, cudaStream_t stream);
void launch_finalize(const DeviceView* views, uint32_t nviews, cudaStream_t stream);

// ---- adjoint of the resolve
struct DiffSetup {
    const float* positions;
    uint32_t vertex_count;
    uint32_t meshlet_count;
    const vkgv_meshlet* meshlets;
    const uint32_t* vertex_indices;
    const uint8_t* tri_indices;
    uint32_t double_sided;
    uint32_t _pad;
    vkgv_vertex* vertices;         // scratch outputs
    vkgv_meshlet_draw* draws;
    float* transform;
    vkgv_primitive* primitive;
    vkgv_material* material;
    const float* colors;           // shading inputs packed for the shade kernel
    const float* uvs;
    float4* vpack;                 // per vertex: (x, y, z, r), (g, b, u, v)
    uint4* tri_verts;              // per visibility id (meshlet << 7 | triangle): its 3 vertex indices
    vkgv_meshlet_cone* cones;      // per meshlet, from the current positions
    uint64_t* cone_table;          // one entry: the address of cones
};

struct DiffArgs {
    const vkgv_meshlet* meshlets;
    const uint32_t* vertex_indices;
    const uint8_t* tri_indices;
    const float* positions;
    const float* colors;
    const float* uvs;
    const float* texture;
    uint32_t tex_w, tex_h;
    float albedo[3];
    float uv_offset[2];
    float uv_scale[2];
    float uv_rotation;
    float scale;
    float* loss;
    float* grad_positions;
    float* grad_colors;
    float* grad_texture;
    // per-vertex / per-texel float4 accumulators (one vector atomic per
    // vertex or texel instead of three), added into the three arrays above
    // by launch_diff_scatter; null where the gradient is not requested
    float4* acc_pos;
    float4* acc_col;
    float4* acc_tex;
    uint32_t vertex_count;
    uint32_t _pad;
    const float4* vpack;           // from DiffSetup
    const uint4* tri_verts;
};

void launch_diff_setup(const DiffSetup& S, cudaStream_t stream);
// Conservative normal cones of every meshlet from the current positions.
void launch_diff_cones(const DiffSetup& S, cudaStream_t stream);
void launch_diff_shade(const DiffArgs& A, const DeviceView* views, uint32_t nviews, uint64_t max_px, bool backward,
                       uint32_t* work, uint32_t sm_count, cudaStream_t stream);
// Adds the float4 accumulators of A into the caller's gradient arrays.
void launch_diff_scatter(const DiffArgs& A, cudaStream_t stream);

// ------------------------------------------------------------------ world
// Device copy of a vkgv_anim_sampler: offsets (in floats) into the pooled
// keyframe array.
struct WorldSampler {
    uint32_t input, output;
    uint32_t input_count, output_count;
    uint32_t interpolation, components;
};

// The node tree's per-frame plan on the device (built once by plan_world).
struct WorldArgs {
    const float* rest;              // 10 floats per node: translation, rotation (x, y, z, w), scale
    const uint32_t* chan_offsets;   // node_count + 1: the node's channels in chans
    const uint2* chans;             // {sampler, path} in application order
    const WorldSampler* samplers;
    const float* keys;              // pooled keyframe times and outputs
    float* local;                   // scratch: T * R * S per node (16 floats)
    const uint32_t* chain_offsets;  // slot_count + 1: the slot's path in chain_nodes
    const uint32_t* chain_nodes;    // root .. node of every transform slot
    const uint32_t* seg_first;      // seg_count + 1: first draw of each (primitive, slot) segment
    const uint2* seg_info;          // {primitive, slot} per segment
    const uint32_t* tile_seg;       // segment of the first draw of every tile of kWorldTile draws
    uint32_t node_count;
    uint32_t slot_count;
    uint32_t seg_count;
    uint32_t draw_count;
    uint32_t tile_count;
};

constexpr uint32_t kWorldTile = 1024;    // draws per k_world_draws block
constexpr uint32_t kWorldThreads = 256;  // threads per k_world_draws block

// Host tables of the plan (uploaded into one device allocation).
struct WorldPlan {
    std::vector<float> rest;
    std::vector<uint32_t> chan_offsets;
    std::vector<uint2> chans;
    std::vector<WorldSampler> samplers;
    std::vector<float> keys;
    std::vector<uint32_t> chain_offsets, chain_nodes;
    std::vector<uint32_t> seg_first;
    std::vector<uint2> seg_info;
    std::vector<uint32_t> tile_seg;
    uint32_t node_count = 0, slot_count = 0, seg_count = 0;
    uint64_t draw_count = 0;
};

// Validates a world description and walks its tree; returns a vkgv_status.
int plan_world(const vkgv_world_desc& desc, WorldPlan& plan, std::string& err);
// k_world_local + k_world_chain: transforms[16 * slot] at `time`.
void launch_world_transforms(const WorldArgs& W, float time, float* transforms, cudaStream_t stream);
// k_world_draws: the MeshletDraw list as 3 words per draw.
void launch_world_draws(const WorldArgs& W, uint32_t* draws, uint32_t sm_count, cudaStream_t stream);

// k_decode_bc: BC1-BC5 blocks -> RGBA8, one thread per texel.
// Sample planes of a JPEG (8-bit, pitch bytes per row) for the colour
// conversion; rx / ry = hmax / h, vmax / v of each component.
struct JpegPlanes {
    const uint8_t* plane[3];
    uint32_t pitch[3], rx[3], ry[3];
    uint32_t width, height, components, rgb;
};

void launch_jpeg_idct(const int16_t* coef, uint32_t blocks_w, uint32_t blocks_h, uint8_t* plane, cudaStream_t stream);
void launch_jpeg_color(const JpegPlanes& P, uint32_t* rgba, cudaStream_t stream);
void launch_decode_bc(const uint8_t* blocks, uint32_t format, uint32_t w, uint32_t h, uint32_t* rgba,
                      cudaStream_t stream);
void launch_decode_bc6h(const uint8_t* blocks, bool is_signed, uint32_t w, uint32_t h, float* rgb,
                        cudaStream_t stream);

}  // namespace vkgv
