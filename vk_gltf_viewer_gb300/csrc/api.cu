// C ABI of libvkgv: context, frame orchestration, stage entry points and
// CUDA-graph capture.  This replaces the per-frame command recording of
// Application::run (src/vk_gltf_viewer/application.cpp:764-1003) and the pass
// initialisation of application.cpp:181-576.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.cuh"

using namespace vkgv;

namespace {

constexpr uint32_t kRing = 4;                 // in-flight frames sharing staging slots
constexpr uint32_t kCountersPerView = 8;      // see DeviceView::counters
constexpr uint32_t kGlobalCounters = 8;       // [0] pass-1 big queue, [1] pass-2 big queue, [2..3] adjoint
                                              // shade work, [4..5] resolve work, [6..7] raster work
constexpr uint32_t kDefaultBigCapacity = 1u << 21;

struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct vkgv_ctx {
    int device = 0;
    uint32_t sm_count = 0;
    vkgv_config cfg{};
    std::string last_error;
    RasterConfig raster{};

    uint32_t* status = nullptr;        // 2 words
    uint32_t* counters = nullptr;      // kGlobalCounters + kCountersPerView * view_cap
    uint32_t view_cap = 0;
    DeviceView* d_views[kRing] = {};
    DeviceView* h_views[kRing] = {};   // pinned staging
    cudaEvent_t ring_ev[kRing] = {};
    bool ring_used[kRing] = {};
    uint32_t ring_pos = 0;

    Scratch survivors;  // per view: capacity draw_count
    Scratch rejected;   // per view: capacity draw_count
    Scratch deferred;   // per view: capacity draw_count
    Scratch reject_samples;  // per view: capacity draw_count (8 B each)
    Scratch diff;       // adjoint: internal raster scene of the differentiable mesh
    Scratch diff_acc;   // adjoint: float4 gradient accumulators (positions, colours, texels)
    Scratch tdet;       // determinant(M) per node transform (vkgv_scene.transform_count)
    Scratch jpeg;       // vkgv_jpeg_to_rgba: coefficient and sample planes
    Scratch mvp;        // view_projection * M per view and node
    BigTri* big = nullptr;
    uint32_t big_cap = 0;
    cudaStream_t capture_stream = nullptr;
    // the final HiZ reduce runs beside the resolve (both only read depth_id)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // Buffers replaced by a larger allocation stay alive until destroy, since
    // a captured graph may still point at them.
    std::vector<void*> retired_dev;
    std::vector<void*> retired_host;
    // GPU stage zones (vkgv_set_profiling)
    bool profile = false;
    bool profile_recorded = false;
    cudaEvent_t zone[VKGV_STAGE_COUNT + 1] = {};
};

struct vkgv_graph {
    vkgv_ctx* ctx = nullptr;
    DeviceView* d_views = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

// A planned node tree: every table in one device allocation.  Updates of one
// world are issued on one stream at a time (they share the local-matrix
// scratch).
struct vkgv_world {
    void* block = nullptr;
    WorldArgs args{};
    uint64_t draw_count = 0;
};

namespace {

int fail(vkgv_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_fail(vkgv_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, VKGV_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VKGV_CUDA(ctx, call)                                   \
    do {                                                       \
        cudaError_t e__ = (call);                              \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call); \
    } while (0)

bool aligned16(uint64_t p) { return (p & 15u) == 0; }

int ensure_scratch(vkgv_ctx* ctx, Scratch& s, size_t bytes, const char* what) {
    if (s.bytes >= bytes) return VKGV_OK;
    if (s.ptr) {
        ctx->retired_dev.push_back(s.ptr);
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = std::max(bytes, size_t(1) << 20);
    if (cudaMalloc(&s.ptr, want) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, VKGV_OUT_OF_MEMORY, std::string("scratch allocation failed: ") + what);
    }
    s.bytes = want;
    return VKGV_OK;
}

int ensure_views(vkgv_ctx* ctx, uint32_t n) {
    if (ctx->view_cap >= n) return VKGV_OK;
    uint32_t cap = std::max<uint32_t>(n, 16);
    for (uint32_t i = 0; i < kRing; ++i) {
        if (ctx->ring_used[i]) VKGV_CUDA(ctx, cudaEventSynchronize(ctx->ring_ev[i]));
        if (ctx->d_views[i]) ctx->retired_dev.push_back(ctx->d_views[i]);
        if (ctx->h_views[i]) ctx->retired_host.push_back(ctx->h_views[i]);
        ctx->d_views[i] = nullptr;
        ctx->h_views[i] = nullptr;
        VKGV_CUDA(ctx, cudaMalloc(&ctx->d_views[i], sizeof(DeviceView) * cap));
        VKGV_CUDA(ctx, cudaMallocHost(&ctx->h_views[i], sizeof(DeviceView) * cap));
        ctx->ring_used[i] = false;
    }
    if (ctx->counters) ctx->retired_dev.push_back(ctx->counters);
    ctx->counters = nullptr;
    VKGV_CUDA(ctx, cudaMalloc(&ctx->counters, sizeof(uint32_t) * (kGlobalCounters + kCountersPerView * cap)));
    VKGV_CUDA(ctx, cudaMemset(ctx->counters, 0, sizeof(uint32_t) * (kGlobalCounters + kCountersPerView * cap)));
    ctx->view_cap = cap;
    return VKGV_OK;
}

int validate_scene(vkgv_ctx* ctx, const vkgv_scene* s) {
    if (!s) return fail(ctx, VKGV_INVALID_ARG, "scene is NULL");
    if (s->meshlet_draw_count >= (1u << VKGV_DRAW_INDEX_BITS))
        return fail(ctx, VKGV_LIMIT_EXCEEDED, "meshlet_draw_count must be < 2^25 (25-bit draw index)");
    if (s->meshlet_draw_count > 0 &&
        (!s->draw_buffer || !s->transform_buffer || !s->primitive_buffer || !s->material_buffer))
        return fail(ctx, VKGV_INVALID_ARG, "scene buffers must be non-NULL");
    if (s->texture_count > 0 && !s->texture_table)
        return fail(ctx, VKGV_INVALID_ARG, "texture_table is NULL with texture_count > 0");
    return VKGV_OK;
}

int validate_pyramid(vkgv_ctx* ctx, const vkgv_pyramid& p, uint32_t w, uint32_t h, const char* which) {
    if (p.levels == 0) return VKGV_OK;
    uint32_t levels = 0;
    uint64_t floats = 0;
    vkgv_pyramid_layout(w, h, &levels, &floats);
    if (!p.data || p.width != (w >> 1) || p.height != (h >> 1) || p.levels != levels)
        return fail(ctx, VKGV_INVALID_ARG,
                    std::string(which) + " pyramid must be (W>>1) x (H>>1) with floor(log2(max(W,H))) levels");
    if (p.data & 3u) return fail(ctx, VKGV_INVALID_ARG, std::string(which) + " pyramid must be 4-byte aligned");
    return VKGV_OK;
}

int validate_view(vkgv_ctx* ctx, const vkgv_view& v, uint32_t flags) {
    if (v.width == 0 || v.height == 0) return fail(ctx, VKGV_INVALID_ARG, "zero-size view");
    if (v.width > VKGV_MAX_VIEW_DIM || v.height > VKGV_MAX_VIEW_DIM)
        return fail(ctx, VKGV_LIMIT_EXCEEDED, "view edge exceeds 8192 pixels");
    if (!v.camera_buffer) return fail(ctx, VKGV_INVALID_ARG, "camera_buffer is NULL");
    if (!v.depth_id || !aligned16(v.depth_id)) return fail(ctx, VKGV_INVALID_ARG, "depth_id must be 16-byte aligned");
    int rc = validate_pyramid(ctx, v.prev_pyramid, v.width, v.height, "prev");
    if (rc) return rc;
    rc = validate_pyramid(ctx, v.pyramid, v.width, v.height, "output");
    if (rc) return rc;
    if ((flags & VKGV_BUILD_PYRAMID) && v.pyramid.levels == 0 && (v.width > 1 || v.height > 1))
        return fail(ctx, VKGV_INVALID_ARG, "VKGV_BUILD_PYRAMID needs an output pyramid");
    if ((flags & (VKGV_RESOLVE_FLAT | VKGV_RESOLVE_TEXTURED)) && !v.color)
        return fail(ctx, VKGV_INVALID_ARG, "resolve requested without a color image");
    if ((flags & VKGV_WRITE_IDS) && !v.visbuffer)
        return fail(ctx, VKGV_INVALID_ARG, "VKGV_WRITE_IDS without a visbuffer image");
    if ((flags & VKGV_WRITE_MOTION) && !v.motion)
        return fail(ctx, VKGV_INVALID_ARG, "VKGV_WRITE_MOTION without a motion image");
    if ((flags & VKGV_RESOLVE_FLAT) && (flags & VKGV_RESOLVE_TEXTURED))
        return fail(ctx, VKGV_INVALID_ARG, "choose one of VKGV_RESOLVE_FLAT and VKGV_RESOLVE_TEXTURED");
    if (v.survivors && !v.survivor_count)
        return fail(ctx, VKGV_INVALID_ARG, "survivors given without survivor_count");
    return VKGV_OK;
}

struct Prepared {
    SceneArgs S;
    uint32_t max_w = 0, max_h = 0;
    uint64_t max_px = 0;
    uint32_t hiz_tx = 1, hiz_ty = 1;  // single-pass HiZ grid (max over views)
    uint32_t hiz_tail = 0;            // its tail's shared-memory floats (max over views)
    float* tdets = nullptr;           // node tables filled by the clear (whole frames only)
    float* mvps = nullptr;
};

// Builds the DeviceView table for `views` into `host` (count n).
int build_views(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* views, uint32_t n, uint32_t flags,
                DeviceView* host, Prepared& P) {
    int rc = validate_scene(ctx, scene);
    if (rc) return rc;
    const uint32_t D = scene->meshlet_draw_count;
    size_t per_view = std::max<size_t>(D, 1) * sizeof(uint32_t);
    rc = ensure_scratch(ctx, ctx->rejected, per_view * n, "rejected lists");
    if (rc) return rc;
    rc = ensure_scratch(ctx, ctx->deferred, per_view * n, "deferred meshlet lists");
    if (rc) return rc;
    const bool two_pass = (flags & VKGV_CULL_TWO_PASS) && (flags & VKGV_CULL_OCCLUSION);
    if (two_pass) {
        rc = ensure_scratch(ctx, ctx->reject_samples, 2 * per_view * n, "pass-1 reject samples");
        if (rc) return rc;
    }
    bool need_surv = false;
    for (uint32_t i = 0; i < n; ++i) need_surv |= views[i].survivors == 0;
    if (need_surv) {
        rc = ensure_scratch(ctx, ctx->survivors, per_view * n, "survivor lists");
        if (rc) return rc;
    }
    if (n > ctx->view_cap) return fail(ctx, VKGV_LIMIT_EXCEEDED, "view table too small");
    P.S.draws = reinterpret_cast<const vkgv_meshlet_draw*>(scene->draw_buffer);
    P.S.transforms = reinterpret_cast<const float*>(scene->transform_buffer);
    P.S.prims = reinterpret_cast<const vkgv_primitive*>(scene->primitive_buffer);
    P.S.mats = reinterpret_cast<const vkgv_material*>(scene->material_buffer);
    P.S.textures = reinterpret_cast<const vkgv_texture*>(scene->texture_table);
    P.S.draw_count = D;
    P.S.texture_count = scene->texture_count;
    P.S.cone_table = reinterpret_cast<const uint64_t*>(scene->cone_table);
    P.S.primitive_count = scene->cone_table ? scene->primitive_count : 0;
    P.S.transform_count = scene->transform_count;
    P.S.tdets = nullptr;
    for (uint32_t i = 0; i < n; ++i) {
        const vkgv_view& v = views[i];
        rc = validate_view(ctx, v, flags);
        if (rc) return rc;
        if (v.survivors && v.survivor_capacity < D)
            return fail(ctx, VKGV_LIMIT_EXCEEDED, "survivor_capacity must be >= meshlet_draw_count");
        DeviceView& d = host[i];
        std::memset(&d, 0, sizeof(d));
        d.cam = reinterpret_cast<const vkgv_camera*>(v.camera_buffer);
        d.w = v.width;
        d.h = v.height;
        d.prev_pyr = reinterpret_cast<const float*>(v.prev_pyramid.data);
        d.prev_w0 = v.prev_pyramid.width;
        d.prev_h0 = v.prev_pyramid.height;
        d.prev_levels = v.prev_pyramid.levels;
        d.pyr = reinterpret_cast<float*>(v.pyramid.data);
        d.pyr_levels = v.pyramid.levels;
        d.depth_id = reinterpret_cast<unsigned long long*>(v.depth_id);
        d.ids = reinterpret_cast<uint32_t*>(v.visbuffer);
        d.rgba = reinterpret_cast<uint32_t*>(v.color);
        d.motion = (flags & VKGV_WRITE_MOTION) ? reinterpret_cast<uint32_t*>(v.motion) : nullptr;
        if (v.survivors) {
            d.survivors = reinterpret_cast<uint32_t*>(v.survivors);
            d.survivor_count = reinterpret_cast<uint32_t*>(v.survivor_count);
            d.survivor_capacity = v.survivor_capacity;
        } else {
            d.survivors = reinterpret_cast<uint32_t*>(ctx->survivors.ptr) + (size_t)i * std::max<uint32_t>(D, 1);
            d.survivor_count = reinterpret_cast<uint32_t*>(v.survivor_count);
            d.survivor_capacity = D;
        }
        d.rejected = reinterpret_cast<uint32_t*>(ctx->rejected.ptr) + (size_t)i * std::max<uint32_t>(D, 1);
        d.deferred = reinterpret_cast<uint32_t*>(ctx->deferred.ptr) + (size_t)i * std::max<uint32_t>(D, 1);
        d.reject_samples = two_pass ? reinterpret_cast<unsigned long long*>(ctx->reject_samples.ptr) +
                                          (size_t)i * std::max<uint32_t>(D, 1)
                                    : nullptr;
        d.counters = ctx->counters + kGlobalCounters + kCountersPerView * i;
        P.max_w = std::max(P.max_w, v.width);
        P.max_h = std::max(P.max_h, v.height);
        if (v.pyramid.levels) {
            uint32_t tx = 1, ty = 1;
            hiz_tiles(v.width, v.height, v.pyramid.levels, &tx, &ty);
            P.hiz_tx = std::max(P.hiz_tx, tx);
            P.hiz_ty = std::max(P.hiz_ty, ty);
            P.hiz_tail = std::max(P.hiz_tail, hiz_tail_floats(v.width, v.height, v.pyramid.levels));
        }
        P.max_px = std::max<uint64_t>(P.max_px, (uint64_t)v.width * v.height);
    }
    return VKGV_OK;
}

// Takes the next staging slot of the view-table ring, waiting until the
// frame that last used it has consumed its table.
int acquire_slot(vkgv_ctx* ctx, int* out_slot, DeviceView** out_dev, DeviceView** out_host) {
    uint32_t slot = ctx->ring_pos;
    ctx->ring_pos = (ctx->ring_pos + 1) % kRing;
    if (ctx->ring_used[slot]) VKGV_CUDA(ctx, cudaEventSynchronize(ctx->ring_ev[slot]));
    *out_slot = (int)slot;
    *out_dev = ctx->d_views[slot];
    *out_host = ctx->h_views[slot];
    return VKGV_OK;
}

int commit_views(vkgv_ctx* ctx, int slot, uint32_t n, cudaStream_t stream) {
    VKGV_CUDA(ctx, cudaMemcpyAsync(ctx->d_views[slot], ctx->h_views[slot], sizeof(DeviceView) * n,
                                   cudaMemcpyHostToDevice, stream));
    return VKGV_OK;
}

int close_slot(vkgv_ctx* ctx, int slot, cudaStream_t stream) {
    VKGV_CUDA(ctx, cudaEventRecord(ctx->ring_ev[slot], stream));
    ctx->ring_used[slot] = true;
    return VKGV_OK;
}

// Records one frame on `stream` for a device view table.  With `zones`,
// zones[i] is recorded at the start of stage i and zones[count] at the end.
void record_frame(vkgv_ctx* ctx, const Prepared& P, const DeviceView* dv, uint32_t n, uint32_t flags,
                  cudaStream_t stream, cudaEvent_t* zones = nullptr) {
    auto zone = [&](int i) {
        if (zones) cudaEventRecord(zones[i], stream);
    };
    uint32_t* gc = ctx->counters;
    const uint32_t T = P.tdets ? P.S.transform_count : 0u;
    zone(0);
    launch_clear(dv, n, (flags & VKGV_SKIP_CLEAR) ? 0 : P.max_px, gc, kGlobalCounters, ctx->sm_count, stream,
                 P.S.transforms, T, P.tdets, P.mvps);
    zone(1);
    launch_cull(P.S, dv, n, flags, 1, ctx->status, ctx->sm_count, stream);
    zone(2);
    RasterLists l1{1, nullptr, nullptr, 0, 4};
    launch_raster(P.S, dv, n, l1, ctx->raster, ctx->big, gc + 0, ctx->big_cap, gc + 6, ctx->status, ctx->sm_count, stream,
                  zones ? zones[3] : nullptr);
    zone(4);
    const bool two = (flags & VKGV_CULL_TWO_PASS) && (flags & VKGV_CULL_OCCLUSION);
    if (two) launch_hiz(dv, n, P.hiz_tx, P.hiz_ty, P.hiz_tail, ctx->status, stream);
    zone(5);
    if (two) launch_cull(P.S, dv, n, flags, 2, ctx->status, ctx->sm_count, stream);
    zone(6);
    if (two) {
        RasterLists l2{2, nullptr, nullptr, 0, 5};
        launch_raster(P.S, dv, n, l2, ctx->raster, ctx->big, gc + 1, ctx->big_cap, gc + 6, ctx->status, ctx->sm_count,
                      stream, zones ? zones[7] : nullptr);
    } else {
        zone(7);
    }
    zone(8);
    // The resolve also writes the survivor totals; without it a small
    // finalise kernel does.
    const bool resolve = (flags & (VKGV_RESOLVE_FLAT | VKGV_RESOLVE_TEXTURED | VKGV_WRITE_IDS | VKGV_WRITE_MOTION)) != 0;
    const bool pyramid = (flags & VKGV_BUILD_PYRAMID) != 0;
    if (pyramid && resolve && !zones) {
        // the pyramid reduce and the resolve both only read the final
        // depth_id: the reduce runs on a side stream beside the resolve
        cudaEventRecord(ctx->fork_ev, stream);
        cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev, 0);
        launch_hiz(dv, n, P.hiz_tx, P.hiz_ty, P.hiz_tail, ctx->status, ctx->side_stream);
        cudaEventRecord(ctx->join_ev, ctx->side_stream);
        launch_resolve(P.S, dv, n, P.max_w, P.max_h, flags, ctx->counters + 4, ctx->sm_count, stream);
        cudaStreamWaitEvent(stream, ctx->join_ev, 0);
    } else {
        if (pyramid) launch_hiz(dv, n, P.hiz_tx, P.hiz_ty, P.hiz_tail, ctx->status, stream);
        zone(9);
        if (resolve) launch_resolve(P.S, dv, n, P.max_w, P.max_h, flags, ctx->counters + 4, ctx->sm_count, stream);
    }
    zone(10);
    if (!resolve) launch_finalize(dv, n, stream);
    zone(11);
}

int check_launch(vkgv_ctx* ctx) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel launch");
    return VKGV_OK;
}

// When the scene gives its node count, a whole frame evaluates each node's
// determinant(M) and each view's view_projection * M once (in the clear
// kernel) instead of once per meshlet draw (raster) or per pixel (resolve).
// Motion-vector frames add prev_view_projection * M after each view's table,
// cone-culled frames the eye in each node's object space (4 floats).
int attach_node_tables(vkgv_ctx* ctx, Prepared& P, DeviceView* host, uint32_t n, uint32_t flags) {
    const size_t T = P.S.transform_count;
    if (T == 0 || P.S.draw_count == 0) return VKGV_OK;
    const bool motion = (flags & VKGV_WRITE_MOTION) != 0;
    const bool eyes = (flags & VKGV_CULL_CONE) && P.S.cone_table;
    const size_t stride = ((motion ? 32 : 16) + (eyes ? 4 : 0)) * T;
    int rc = ensure_scratch(ctx, ctx->tdet, sizeof(float) * T, "node determinants");
    if (rc) return rc;
    rc = ensure_scratch(ctx, ctx->mvp, sizeof(float) * stride * n, "per-view node matrices");
    if (rc) return rc;
    P.tdets = static_cast<float*>(ctx->tdet.ptr);
    P.mvps = static_cast<float*>(ctx->mvp.ptr);
    P.S.tdets = P.tdets;
    for (uint32_t i = 0; i < n; ++i) {
        host[i].mvps = P.mvps + stride * i;
        host[i].prev_mvps = motion ? P.mvps + stride * i + 16 * T : nullptr;
        host[i].eyes = eyes ? reinterpret_cast<const float4*>(P.mvps + stride * i + (motion ? 32 : 16) * T) : nullptr;
    }
    return VKGV_OK;
}

int two_pass_needs_pyramid(vkgv_ctx* ctx, const vkgv_view* views, uint32_t n, uint32_t flags) {
    if ((flags & VKGV_CULL_TWO_PASS) && (flags & VKGV_CULL_OCCLUSION))
        for (uint32_t i = 0; i < n; ++i)
            if (views[i].prev_pyramid.levels && !views[i].pyramid.levels)
                return fail(ctx, VKGV_INVALID_ARG, "two-pass culling needs an output pyramid");
    return VKGV_OK;
}

}  // namespace

extern "C" {

int vkgv_create(const vkgv_config* config, vkgv_ctx** out_ctx) {
    if (!out_ctx) return VKGV_INVALID_ARG;
    *out_ctx = nullptr;
    vkgv_ctx* ctx = new (std::nothrow) vkgv_ctx();
    if (!ctx) return VKGV_OUT_OF_MEMORY;
    if (config) ctx->cfg = *config;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        delete ctx;
        return VKGV_CUDA_ERROR;
    }
    if (ctx->cfg.device < 0 || ctx->cfg.device >= ndev) {
        delete ctx;
        return VKGV_INVALID_ARG;
    }
    ctx->device = ctx->cfg.device;
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        delete ctx;
        return VKGV_CUDA_ERROR;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    ctx->sm_count = (uint32_t)std::max(sms, 1);
    uint32_t bin = ctx->cfg.bin_size ? ctx->cfg.bin_size : 32;
    if (bin != 8 && bin != 16 && bin != 32 && bin != 64) {
        delete ctx;
        return VKGV_INVALID_ARG;
    }
    uint32_t mpc = ctx->cfg.meshlets_per_cta ? ctx->cfg.meshlets_per_cta : 4;
    if (mpc != 1 && mpc != 2 && mpc != 4 && mpc != 8) {
        delete ctx;
        return VKGV_INVALID_ARG;
    }
    ctx->raster.chunk = bin;
    ctx->raster.small_area = bin * bin > 64 ? 64 : bin * bin;
    ctx->raster.warps_per_cta = mpc;
    ctx->raster.blocks_per_view = 0;
    ctx->big_cap = ctx->cfg.big_triangle_capacity ? ctx->cfg.big_triangle_capacity : kDefaultBigCapacity;
    bool ok = cudaMalloc(&ctx->status, 2 * sizeof(uint32_t)) == cudaSuccess &&
              cudaMemset(ctx->status, 0, 2 * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&ctx->big, sizeof(BigTri) * (size_t)ctx->big_cap) == cudaSuccess &&
              cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) == cudaSuccess;
    for (uint32_t i = 0; ok && i < kRing; ++i)
        ok = cudaEventCreateWithFlags(&ctx->ring_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        vkgv_destroy(ctx);
        return VKGV_OUT_OF_MEMORY;
    }
    if (ensure_views(ctx, 16) != VKGV_OK) {
        vkgv_destroy(ctx);
        return VKGV_OUT_OF_MEMORY;
    }
    *out_ctx = ctx;
    return VKGV_OK;
}

int vkgv_destroy(vkgv_ctx* ctx) {
    if (!ctx) return VKGV_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (uint32_t i = 0; i < kRing; ++i) {
        if (ctx->d_views[i]) cudaFree(ctx->d_views[i]);
        if (ctx->h_views[i]) cudaFreeHost(ctx->h_views[i]);
        if (ctx->ring_ev[i]) cudaEventDestroy(ctx->ring_ev[i]);
    }
    if (ctx->counters) cudaFree(ctx->counters);
    if (ctx->status) cudaFree(ctx->status);
    if (ctx->big) cudaFree(ctx->big);
    if (ctx->survivors.ptr) cudaFree(ctx->survivors.ptr);
    if (ctx->rejected.ptr) cudaFree(ctx->rejected.ptr);
    if (ctx->deferred.ptr) cudaFree(ctx->deferred.ptr);
    if (ctx->reject_samples.ptr) cudaFree(ctx->reject_samples.ptr);
    if (ctx->diff.ptr) cudaFree(ctx->diff.ptr);
    if (ctx->diff_acc.ptr) cudaFree(ctx->diff_acc.ptr);
    if (ctx->tdet.ptr) cudaFree(ctx->tdet.ptr);
    if (ctx->jpeg.ptr) cudaFree(ctx->jpeg.ptr);
    if (ctx->mvp.ptr) cudaFree(ctx->mvp.ptr);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    for (uint32_t i = 0; i <= VKGV_STAGE_COUNT; ++i)
        if (ctx->zone[i]) cudaEventDestroy(ctx->zone[i]);
    for (void* p : ctx->retired_dev) cudaFree(p);
    for (void* p : ctx->retired_host) cudaFreeHost(p);
    delete ctx;
    return VKGV_OK;
}

const char* vkgv_last_error(const vkgv_ctx* ctx) {
    if (!ctx) return "null context";
    return ctx->last_error.c_str();
}

int vkgv_device_status(vkgv_ctx* ctx, uint32_t* out_code, uint32_t* out_detail) {
    if (!ctx || !out_code || !out_detail) return VKGV_INVALID_ARG;
    uint32_t h[2] = {0, 0};
    VKGV_CUDA(ctx, cudaMemcpy(h, ctx->status, sizeof(h), cudaMemcpyDeviceToHost));
    VKGV_CUDA(ctx, cudaMemset(ctx->status, 0, sizeof(h)));
    *out_code = h[0];
    *out_detail = h[1];
    return VKGV_OK;
}

int vkgv_frame(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* views, uint32_t view_count, uint32_t flags,
               void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!views || view_count == 0) return fail(ctx, VKGV_INVALID_ARG, "no views");
    if (view_count > 65535u) return fail(ctx, VKGV_LIMIT_EXCEEDED, "at most 65535 views per frame");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    int rc = two_pass_needs_pyramid(ctx, views, view_count, flags);
    if (rc) return rc;
    rc = ensure_views(ctx, view_count);
    if (rc) return rc;
    DeviceView *dv, *hv;
    int slot = 0;
    rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, scene, views, view_count, flags, hv, P);
    if (rc) return rc;
    rc = attach_node_tables(ctx, P, hv, view_count, flags);
    if (rc) return rc;
    rc = commit_views(ctx, slot, view_count, stream);
    if (rc) return rc;
    record_frame(ctx, P, dv, view_count, flags, stream, ctx->profile ? ctx->zone : nullptr);
    if (ctx->profile) ctx->profile_recorded = true;
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

int vkgv_set_profiling(vkgv_ctx* ctx, int32_t enable) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (enable && !ctx->zone[0])
        for (uint32_t i = 0; i <= VKGV_STAGE_COUNT; ++i) VKGV_CUDA(ctx, cudaEventCreate(&ctx->zone[i]));
    ctx->profile = enable != 0;
    ctx->profile_recorded = false;
    return VKGV_OK;
}

int vkgv_stage_times(vkgv_ctx* ctx, float* out_ms, uint32_t count) {
    if (!ctx || !out_ms) return VKGV_INVALID_ARG;
    if (!ctx->profile_recorded) return fail(ctx, VKGV_INVALID_ARG, "no profiled frame recorded");
    VKGV_CUDA(ctx, cudaEventSynchronize(ctx->zone[VKGV_STAGE_COUNT]));
    for (uint32_t i = 0; i < count && i < VKGV_STAGE_COUNT; ++i) {
        float ms = 0.f;
        VKGV_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->zone[i], ctx->zone[i + 1]));
        out_ms[i] = ms;
    }
    return VKGV_OK;
}

int vkgv_clear(vkgv_ctx* ctx, const vkgv_view* view, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!view) return fail(ctx, VKGV_INVALID_ARG, "view is NULL");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    vkgv_scene empty{};
    DeviceView *dv, *hv;
    int slot = 0;
    int rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, &empty, view, 1, 0, hv, P);
    if (rc) return rc;
    rc = commit_views(ctx, slot, 1, stream);
    if (rc) return rc;
    launch_clear(dv, 1, P.max_px, ctx->counters, kGlobalCounters, ctx->sm_count, stream);
    launch_finalize(dv, 1, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

int vkgv_cull(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view, uint32_t flags, uint32_t pass,
              void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!view) return fail(ctx, VKGV_INVALID_ARG, "view is NULL");
    if (pass != 1 && pass != 2) return fail(ctx, VKGV_INVALID_ARG, "pass must be 1 or 2");
    if (!view->survivors) return fail(ctx, VKGV_INVALID_ARG, "vkgv_cull needs view->survivors");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    DeviceView *dv, *hv;
    int slot = 0;
    int rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, scene, view, 1,
                     flags & ~(VKGV_BUILD_PYRAMID | VKGV_RESOLVE_FLAT | VKGV_RESOLVE_TEXTURED | VKGV_WRITE_IDS |
                               VKGV_WRITE_MOTION),
                     hv, P);
    if (rc) return rc;
    rc = commit_views(ctx, slot, 1, stream);
    if (rc) return rc;
    launch_cull(P.S, dv, 1, flags, pass, ctx->status, ctx->sm_count, stream);
    launch_finalize(dv, 1, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

int vkgv_raster(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view, uint64_t draw_list,
                uint64_t draw_count, uint32_t first, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!view) return fail(ctx, VKGV_INVALID_ARG, "view is NULL");
    if ((draw_list == 0) != (draw_count == 0))
        return fail(ctx, VKGV_INVALID_ARG, "draw_list and draw_count must both be set or both be 0");
    if (!draw_list && (!view->survivors || !view->survivor_count))
        return fail(ctx, VKGV_INVALID_ARG, "vkgv_raster without a list needs view->survivors and survivor_count");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    DeviceView *dv, *hv;
    int slot = 0;
    int rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, scene, view, 1, 0, hv, P);
    if (rc) return rc;
    rc = commit_views(ctx, slot, 1, stream);
    if (rc) return rc;
    RasterLists l{0, draw_list ? reinterpret_cast<const uint32_t*>(draw_list) : reinterpret_cast<const uint32_t*>(view->survivors),
                  draw_count ? reinterpret_cast<const uint32_t*>(draw_count)
                             : reinterpret_cast<const uint32_t*>(view->survivor_count),
                  first, 6};
    // big-queue counter and the view's deferred-list counter start at zero
    VKGV_CUDA(ctx, cudaMemsetAsync(ctx->counters, 0, sizeof(uint32_t), stream));
    VKGV_CUDA(ctx, cudaMemsetAsync(ctx->counters + kGlobalCounters + 6, 0, sizeof(uint32_t), stream));
    launch_raster(P.S, dv, 1, l, ctx->raster, ctx->big, ctx->counters, ctx->big_cap, ctx->counters + 6, ctx->status,
                  ctx->sm_count, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

int vkgv_hiz_reduce(vkgv_ctx* ctx, const vkgv_view* view, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!view) return fail(ctx, VKGV_INVALID_ARG, "view is NULL");
    if (view->pyramid.levels == 0) return fail(ctx, VKGV_INVALID_ARG, "view has no output pyramid");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    vkgv_scene empty{};
    DeviceView *dv, *hv;
    int slot = 0;
    int rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, &empty, view, 1, VKGV_BUILD_PYRAMID, hv, P);
    if (rc) return rc;
    rc = commit_views(ctx, slot, 1, stream);
    if (rc) return rc;
    launch_hiz(dv, 1, P.hiz_tx, P.hiz_ty, P.hiz_tail, ctx->status, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

int vkgv_resolve(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* view, uint32_t flags, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!view) return fail(ctx, VKGV_INVALID_ARG, "view is NULL");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    DeviceView *dv, *hv;
    int slot = 0;
    int rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    Prepared P;
    rc = build_views(ctx, scene, view, 1,
                     flags & (VKGV_RESOLVE_FLAT | VKGV_RESOLVE_TEXTURED | VKGV_WRITE_IDS | VKGV_WRITE_MOTION), hv, P);
    if (rc) return rc;
    rc = commit_views(ctx, slot, 1, stream);
    if (rc) return rc;
    launch_resolve(P.S, dv, 1, P.max_w, P.max_h, flags, ctx->counters + 4, ctx->sm_count, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}


int vkgv_decode_bc(vkgv_ctx* ctx, uint32_t format, uint64_t blocks, uint32_t width, uint32_t height,
                   uint64_t rgba_out, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (format < VKGV_BC1 || (format > VKGV_BC1_OPAQUE && format != VKGV_BC7))
        return fail(ctx, VKGV_INVALID_ARG, "unknown block format");
    if (width == 0 || height == 0) return VKGV_OK;
    if (width > 16384 || height > 16384) return fail(ctx, VKGV_LIMIT_EXCEEDED, "texture edge exceeds 16384");
    const uint64_t block_align = (format == VKGV_BC1 || format == VKGV_BC4 || format == VKGV_BC1_OPAQUE) ? 8u : 16u;
    if (!blocks || !rgba_out || (blocks & (block_align - 1)) || (rgba_out & 3u))
        return fail(ctx, VKGV_INVALID_ARG, "blocks must be aligned to the block size and rgba_out to 4 bytes");
    launch_decode_bc(reinterpret_cast<const uint8_t*>(blocks), format, width, height,
                     reinterpret_cast<uint32_t*>(rgba_out), reinterpret_cast<cudaStream_t>(stream_));
    return check_launch(ctx);
}

int vkgv_decode_bc6h(vkgv_ctx* ctx, uint32_t format, uint64_t blocks, uint32_t width, uint32_t height,
                     uint64_t rgb_out, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (format != VKGV_BC6H_UF16 && format != VKGV_BC6H_SF16) return fail(ctx, VKGV_INVALID_ARG, "not a BC6H format");
    if (width == 0 || height == 0) return VKGV_OK;
    if (width > 16384 || height > 16384) return fail(ctx, VKGV_LIMIT_EXCEEDED, "texture edge exceeds 16384");
    if (!blocks || !rgb_out || (blocks & 15u) || (rgb_out & 3u))
        return fail(ctx, VKGV_INVALID_ARG, "blocks must be 16-byte aligned and rgb_out 4-byte aligned");
    launch_decode_bc6h(reinterpret_cast<const uint8_t*>(blocks), format == VKGV_BC6H_SF16, width, height,
                       reinterpret_cast<float*>(rgb_out), reinterpret_cast<cudaStream_t>(stream_));
    return check_launch(ctx);
}

int vkgv_jpeg_to_rgba(vkgv_ctx* ctx, const vkgv_jpeg* jpeg, uint64_t rgba_out, void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    vkgv_jpeg_info I;
    if (!jpeg || vkgv_jpeg_get_info(jpeg, &I) != VKGV_OK) return fail(ctx, VKGV_INVALID_ARG, "jpeg must be non-NULL");
    if (!rgba_out || (rgba_out & 3u)) return fail(ctx, VKGV_INVALID_ARG, "rgba_out must be non-NULL and 4-byte aligned");
    const auto stream = reinterpret_cast<cudaStream_t>(stream_);
    // per component: its coefficient plane, then its sample plane
    size_t coef_at[3], plane_at[3], off = 0;
    for (uint32_t c = 0; c < I.components; ++c) {
        const size_t blocks = size_t(I.blocks_w[c]) * I.blocks_h[c];
        coef_at[c] = off;
        off += (blocks * 128 + 255) & ~size_t(255);
        plane_at[c] = off;
        off += (blocks * 64 + 255) & ~size_t(255);
    }
    int rc = ensure_scratch(ctx, ctx->jpeg, off, "JPEG planes");
    if (rc) return rc;
    auto* base = static_cast<uint8_t*>(ctx->jpeg.ptr);
    JpegPlanes P{};
    for (uint32_t c = 0; c < I.components; ++c) {
        const int16_t* host = nullptr;
        if (vkgv_jpeg_get_coefficients(jpeg, c, &host) != VKGV_OK) return fail(ctx, VKGV_INVALID_ARG, "bad JPEG");
        const size_t blocks = size_t(I.blocks_w[c]) * I.blocks_h[c];
        // pageable source: returns once the data is staged, so the caller may free it
        VKGV_CUDA(ctx, cudaMemcpyAsync(base + coef_at[c], host, blocks * 128, cudaMemcpyHostToDevice, stream));
        launch_jpeg_idct(reinterpret_cast<const int16_t*>(base + coef_at[c]), I.blocks_w[c], I.blocks_h[c],
                         base + plane_at[c], stream);
        P.plane[c] = base + plane_at[c];
        P.pitch[c] = I.blocks_w[c] * 8;
        P.rx[c] = I.hmax / I.h[c];
        P.ry[c] = I.vmax / I.v[c];
    }
    P.width = I.width;
    P.height = I.height;
    P.components = I.components;
    P.rgb = I.rgb;
    launch_jpeg_color(P, reinterpret_cast<uint32_t*>(rgba_out), stream);
    return check_launch(ctx);
}

int vkgv_world_create(vkgv_ctx* ctx, const vkgv_world_desc* desc, vkgv_world** out_world) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!desc || !out_world) return fail(ctx, VKGV_INVALID_ARG, "desc and out_world must be non-NULL");
    *out_world = nullptr;
    WorldPlan P;
    std::string err;
    int rc = plan_world(*desc, P, err);
    if (rc) return fail(ctx, rc, err);
    // one allocation, each table 16-byte aligned
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 15) & ~size_t(15);
        return at;
    };
    const size_t o_rest = place(sizeof(float) * P.rest.size());
    const size_t o_coff = place(sizeof(uint32_t) * P.chan_offsets.size());
    const size_t o_chans = place(sizeof(uint2) * P.chans.size());
    const size_t o_samp = place(sizeof(WorldSampler) * P.samplers.size());
    const size_t o_keys = place(sizeof(float) * P.keys.size());
    const size_t o_local = place(sizeof(float) * 16 * (size_t)P.node_count);
    const size_t o_choff = place(sizeof(uint32_t) * P.chain_offsets.size());
    const size_t o_chain = place(sizeof(uint32_t) * P.chain_nodes.size());
    const size_t o_sfirst = place(sizeof(uint32_t) * P.seg_first.size());
    const size_t o_sinfo = place(sizeof(uint2) * P.seg_info.size());
    const size_t o_tiles = place(sizeof(uint32_t) * P.tile_seg.size());
    vkgv_world* w = new (std::nothrow) vkgv_world();
    if (!w) return fail(ctx, VKGV_OUT_OF_MEMORY, "world allocation failed");
    if (cudaMalloc(&w->block, std::max<size_t>(off, 16)) != cudaSuccess) {
        cudaGetLastError();
        delete w;
        return fail(ctx, VKGV_OUT_OF_MEMORY, "world device tables");
    }
    char* b = static_cast<char*>(w->block);
    auto put = [&](size_t at, const void* src, size_t bytes) {
        return bytes ? cudaMemcpy(b + at, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = put(o_rest, P.rest.data(), sizeof(float) * P.rest.size());
    if (e == cudaSuccess) e = put(o_coff, P.chan_offsets.data(), sizeof(uint32_t) * P.chan_offsets.size());
    if (e == cudaSuccess) e = put(o_chans, P.chans.data(), sizeof(uint2) * P.chans.size());
    if (e == cudaSuccess) e = put(o_samp, P.samplers.data(), sizeof(WorldSampler) * P.samplers.size());
    if (e == cudaSuccess) e = put(o_keys, P.keys.data(), sizeof(float) * P.keys.size());
    if (e == cudaSuccess) e = put(o_choff, P.chain_offsets.data(), sizeof(uint32_t) * P.chain_offsets.size());
    if (e == cudaSuccess) e = put(o_chain, P.chain_nodes.data(), sizeof(uint32_t) * P.chain_nodes.size());
    if (e == cudaSuccess) e = put(o_sfirst, P.seg_first.data(), sizeof(uint32_t) * P.seg_first.size());
    if (e == cudaSuccess) e = put(o_sinfo, P.seg_info.data(), sizeof(uint2) * P.seg_info.size());
    if (e == cudaSuccess) e = put(o_tiles, P.tile_seg.data(), sizeof(uint32_t) * P.tile_seg.size());
    if (e != cudaSuccess) {
        cudaFree(w->block);
        delete w;
        return cuda_fail(ctx, e, "world upload");
    }
    WorldArgs& A = w->args;
    A.rest = reinterpret_cast<const float*>(b + o_rest);
    A.chan_offsets = reinterpret_cast<const uint32_t*>(b + o_coff);
    A.chans = reinterpret_cast<const uint2*>(b + o_chans);
    A.samplers = reinterpret_cast<const WorldSampler*>(b + o_samp);
    A.keys = reinterpret_cast<const float*>(b + o_keys);
    A.local = reinterpret_cast<float*>(b + o_local);
    A.chain_offsets = reinterpret_cast<const uint32_t*>(b + o_choff);
    A.chain_nodes = reinterpret_cast<const uint32_t*>(b + o_chain);
    A.seg_first = reinterpret_cast<const uint32_t*>(b + o_sfirst);
    A.seg_info = reinterpret_cast<const uint2*>(b + o_sinfo);
    A.tile_seg = reinterpret_cast<const uint32_t*>(b + o_tiles);
    A.tile_count = (uint32_t)P.tile_seg.size();
    A.node_count = P.node_count;
    A.slot_count = P.slot_count;
    A.seg_count = P.seg_count;
    A.draw_count = (uint32_t)P.draw_count;
    w->draw_count = P.draw_count;
    *out_world = w;
    return VKGV_OK;
}

int vkgv_world_destroy(vkgv_world* world) {
    if (!world) return VKGV_INVALID_ARG;
    if (world->block) cudaFree(world->block);
    delete world;
    return VKGV_OK;
}

int vkgv_world_info(const vkgv_world* world, uint32_t* out_transform_count, uint64_t* out_draw_count) {
    if (!world) return VKGV_INVALID_ARG;
    if (out_transform_count) *out_transform_count = world->args.slot_count;
    if (out_draw_count) *out_draw_count = world->draw_count;
    return VKGV_OK;
}

int vkgv_world_update_transforms(vkgv_ctx* ctx, vkgv_world* world, float animation_time, uint64_t transform_buffer,
                                 void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!world) return fail(ctx, VKGV_INVALID_ARG, "world is NULL");
    if (world->args.slot_count && (!transform_buffer || !aligned16(transform_buffer)))
        return fail(ctx, VKGV_INVALID_ARG, "transform_buffer must be 16-byte aligned");
    launch_world_transforms(world->args, animation_time, reinterpret_cast<float*>(transform_buffer),
                            reinterpret_cast<cudaStream_t>(stream_));
    return check_launch(ctx);
}

int vkgv_world_build_draws(vkgv_ctx* ctx, vkgv_world* world, uint64_t draw_buffer, uint64_t capacity,
                           void* stream_) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!world) return fail(ctx, VKGV_INVALID_ARG, "world is NULL");
    if (capacity < world->draw_count) return fail(ctx, VKGV_LIMIT_EXCEEDED, "draw buffer capacity below the draw count");
    if (world->draw_count && (!draw_buffer || !aligned16(draw_buffer)))
        return fail(ctx, VKGV_INVALID_ARG, "draw_buffer must be 16-byte aligned");
    launch_world_draws(world->args, reinterpret_cast<uint32_t*>(draw_buffer), ctx->sm_count,
                       reinterpret_cast<cudaStream_t>(stream_));
    return check_launch(ctx);
}

}  // extern "C"

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// The adjoint's launch plan: the internal raster scene built from the
// current positions (identity node transform, one draw per meshlet), the
// per-view device descriptors and the shading arguments.
struct DiffPlan {
    DiffSetup S{};
    DiffArgs A{};
    Prepared P;
    std::vector<DeviceView> views;
    size_t acc_bytes = 0;  // float4 accumulators to zero before a backward pass
    uint32_t cone_mode = 0;
};

int diff_prepare(vkgv_ctx* ctx, const vkgv_diff_scene* ds, const vkgv_diff_view* views, uint32_t n, bool backward,
                 float scale, uint64_t loss, uint64_t gpos, uint64_t gcol, uint64_t gtex, DiffPlan& D) {
    if (!ctx) return VKGV_INVALID_ARG;
    if (!ds || !views || n == 0) return fail(ctx, VKGV_INVALID_ARG, "adjoint: scene and views are required");
    if (!ds->meshlet_buffer || !ds->vertex_index_buffer || !ds->primitive_index_buffer || !ds->positions ||
        !ds->colors || !ds->uvs || !ds->texture || ds->vertex_count == 0 || ds->tex_width == 0 || ds->tex_height == 0)
        return fail(ctx, VKGV_INVALID_ARG, "adjoint: incomplete scene");
    if (ds->cone_mode > 2) return fail(ctx, VKGV_INVALID_ARG, "adjoint: cone_mode must be 0, 1 or 2");
    if (ds->meshlet_count >= (1u << VKGV_DRAW_INDEX_BITS))
        return fail(ctx, VKGV_LIMIT_EXCEEDED, "adjoint: meshlet_count must be < 2^25");
    if (n > 65535u) return fail(ctx, VKGV_LIMIT_EXCEEDED, "at most 65535 views per call");
    const size_t V = ds->vertex_count, M = ds->meshlet_count;
    const size_t off_draws = align256(sizeof(vkgv_vertex) * V);
    const size_t off_xf = off_draws + align256(sizeof(vkgv_meshlet_draw) * std::max<size_t>(M, 1));
    const size_t off_prim = off_xf + 256, off_mat = off_prim + 256, off_vpack = off_mat + 256;
    const size_t off_tri = off_vpack + align256(2 * sizeof(float4) * V);
    const size_t off_cones = off_tri + align256(sizeof(uint4) * (std::max<size_t>(M, 1) << VKGV_TRIANGLE_BITS));
    const size_t off_cone_table = off_cones + align256(sizeof(vkgv_meshlet_cone) * std::max<size_t>(M, 1));
    const size_t total = off_cone_table + 256;
    int rc = ensure_scratch(ctx, ctx->diff, total, "adjoint scene");
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->diff.ptr);
    DiffSetup& S = D.S;
    S.positions = reinterpret_cast<const float*>(ds->positions);
    S.vertex_count = ds->vertex_count;
    S.meshlet_count = ds->meshlet_count;
    S.meshlets = reinterpret_cast<const vkgv_meshlet*>(ds->meshlet_buffer);
    S.vertex_indices = reinterpret_cast<const uint32_t*>(ds->vertex_index_buffer);
    S.tri_indices = reinterpret_cast<const uint8_t*>(ds->primitive_index_buffer);
    S.double_sided = ds->double_sided;
    S.vertices = reinterpret_cast<vkgv_vertex*>(base);
    S.draws = reinterpret_cast<vkgv_meshlet_draw*>(base + off_draws);
    S.transform = reinterpret_cast<float*>(base + off_xf);
    S.primitive = reinterpret_cast<vkgv_primitive*>(base + off_prim);
    S.material = reinterpret_cast<vkgv_material*>(base + off_mat);
    S.colors = reinterpret_cast<const float*>(ds->colors);
    S.uvs = reinterpret_cast<const float*>(ds->uvs);
    S.vpack = reinterpret_cast<float4*>(base + off_vpack);
    S.tri_verts = reinterpret_cast<uint4*>(base + off_tri);
    S.cones = reinterpret_cast<vkgv_meshlet_cone*>(base + off_cones);
    S.cone_table = reinterpret_cast<uint64_t*>(base + off_cone_table);
    vkgv_scene scene{};
    scene.draw_buffer = reinterpret_cast<uint64_t>(S.draws);
    scene.transform_buffer = reinterpret_cast<uint64_t>(S.transform);
    scene.primitive_buffer = reinterpret_cast<uint64_t>(S.primitive);
    scene.material_buffer = reinterpret_cast<uint64_t>(S.material);
    scene.meshlet_draw_count = ds->meshlet_count;
    // normal cones rebuilt from the current positions on every pass
    scene.cone_table = reinterpret_cast<uint64_t>(S.cone_table);
    scene.primitive_count = 1;
    std::vector<vkgv_view> vv(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (backward && !views[i].target && !views[i].grad_rgb)
            return fail(ctx, VKGV_INVALID_ARG, "adjoint: backward needs a target or grad_rgb per view");
        vv[i] = vkgv_view{};
        vv[i].camera_buffer = views[i].camera_buffer;
        vv[i].width = views[i].width;
        vv[i].height = views[i].height;
        vv[i].depth_id = views[i].depth_id;
    }
    rc = ensure_views(ctx, n);
    if (rc) return rc;
    D.views.assign(n, DeviceView{});
    rc = build_views(ctx, &scene, vv.data(), n, 0, D.views.data(), D.P);
    if (rc) return rc;
    for (uint32_t i = 0; i < n; ++i) {
        D.views[i].diff_rgb = reinterpret_cast<float*>(views[i].rgb);
        D.views[i].diff_target = reinterpret_cast<const float*>(views[i].target);
        D.views[i].diff_grad = reinterpret_cast<const float*>(views[i].grad_rgb);
    }
    DiffArgs& A = D.A;
    A.meshlets = S.meshlets;
    A.vertex_indices = S.vertex_indices;
    A.tri_indices = S.tri_indices;
    A.positions = S.positions;
    A.colors = reinterpret_cast<const float*>(ds->colors);
    A.uvs = reinterpret_cast<const float*>(ds->uvs);
    A.texture = reinterpret_cast<const float*>(ds->texture);
    A.tex_w = ds->tex_width;
    A.tex_h = ds->tex_height;
    for (int k = 0; k < 3; ++k) A.albedo[k] = ds->albedo[k];
    for (int k = 0; k < 2; ++k) {
        A.uv_offset[k] = ds->uv_offset[k];
        A.uv_scale[k] = ds->uv_scale[k];
    }
    A.uv_rotation = ds->uv_rotation;
    A.scale = scale;
    A.loss = reinterpret_cast<float*>(loss);
    A.grad_positions = reinterpret_cast<float*>(gpos);
    A.grad_colors = reinterpret_cast<float*>(gcol);
    A.grad_texture = reinterpret_cast<float*>(gtex);
    D.cone_mode = ds->cone_mode;
    A.vertex_count = ds->vertex_count;
    A.vpack = S.vpack;
    A.tri_verts = S.tri_verts;
    if (backward) {
        const size_t nv = gpos ? V : 0, nc = gcol ? V : 0, nt = gtex ? (size_t)ds->tex_width * ds->tex_height : 0;
        D.acc_bytes = sizeof(float4) * (nv + nc + nt);
        if (D.acc_bytes) {
            rc = ensure_scratch(ctx, ctx->diff_acc, D.acc_bytes, "adjoint accumulators");
            if (rc) return rc;
            float4* acc = static_cast<float4*>(ctx->diff_acc.ptr);
            A.acc_pos = gpos ? acc : nullptr;
            A.acc_col = gcol ? acc + nv : nullptr;
            A.acc_tex = gtex ? acc + nv + nc : nullptr;
        }
    }
    return VKGV_OK;
}

// One pass of the adjoint over device view descriptors dv: vertex records
// and meshlet normal cones from the current positions, visibility
// recomputed (clear, cone-only cull: the builder's meshlet bounds do not
// follow moving vertices, raster), then the shading kernel forward or
// backward.
void diff_record(vkgv_ctx* ctx, const DiffPlan& D, const DeviceView* dv, uint32_t n, bool backward,
                 cudaStream_t stream) {
    launch_diff_setup(D.S, stream);
    // The cone pass has a fixed cost of a few tens of microseconds; it pays
    // once the pass rasterises enough meshlet-views (measured: 220 meshlets
    // x 64 views ran 5% slower with it, 14k x 512 ran 13% faster).
    const bool cones = D.cone_mode == 1 || (D.cone_mode == 0 && (uint64_t)D.S.meshlet_count * n >= (1ull << 20));
    if (cones) launch_diff_cones(D.S, stream);
    launch_clear(dv, n, D.P.max_px, ctx->counters, kGlobalCounters, ctx->sm_count, stream);
    launch_cull(D.P.S, dv, n, cones ? (uint32_t)VKGV_CULL_CONE : 0u, 1, ctx->status, ctx->sm_count, stream);
    RasterLists l1{1, nullptr, nullptr, 0, 4};
    launch_raster(D.P.S, dv, n, l1, ctx->raster, ctx->big, ctx->counters + 0, ctx->big_cap, ctx->counters + 6, ctx->status,
                  ctx->sm_count, stream);
    if (backward && D.acc_bytes) cudaMemsetAsync(ctx->diff_acc.ptr, 0, D.acc_bytes, stream);
    launch_diff_shade(D.A, dv, n, D.P.max_px, backward, ctx->counters + 2, ctx->sm_count, stream);
    if (backward) launch_diff_scatter(D.A, stream);
}

int diff_run(vkgv_ctx* ctx, const vkgv_diff_scene* ds, const vkgv_diff_view* views, uint32_t n, bool backward,
             float scale, uint64_t loss, uint64_t gpos, uint64_t gcol, uint64_t gtex, void* stream_) {
    DiffPlan D;
    int rc = diff_prepare(ctx, ds, views, n, backward, scale, loss, gpos, gcol, gtex, D);
    if (rc) return rc;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    DeviceView *dv, *hv;
    int slot = 0;
    rc = acquire_slot(ctx, &slot, &dv, &hv);
    if (rc) return rc;
    std::memcpy(hv, D.views.data(), sizeof(DeviceView) * n);
    rc = commit_views(ctx, slot, n, stream);
    if (rc) return rc;
    diff_record(ctx, D, dv, n, backward, stream);
    rc = check_launch(ctx);
    if (rc) return rc;
    return close_slot(ctx, slot, stream);
}

}  // namespace

extern "C" {

int vkgv_diff_forward(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views, uint32_t view_count,
                      void* stream) {
    return diff_run(ctx, scene, views, view_count, false, 0.0f, 0, 0, 0, 0, stream);
}

int vkgv_diff_backward(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views, uint32_t view_count,
                       float scale, uint64_t loss, uint64_t grad_positions, uint64_t grad_colors,
                       uint64_t grad_texture, void* stream) {
    return diff_run(ctx, scene, views, view_count, true, scale, loss, grad_positions, grad_colors, grad_texture,
                    stream);
}

int vkgv_diff_graph_capture(vkgv_ctx* ctx, const vkgv_diff_scene* scene, const vkgv_diff_view* views,
                            uint32_t view_count, uint32_t passes, float scale, uint64_t loss, uint64_t grad_positions,
                            uint64_t grad_colors, uint64_t grad_texture, vkgv_graph** out_graph) {
    if (!ctx || !out_graph) return VKGV_INVALID_ARG;
    *out_graph = nullptr;
    const uint32_t known = VKGV_DIFF_ZERO_GRADS | VKGV_DIFF_FORWARD | VKGV_DIFF_BACKWARD;
    if (passes == 0 || (passes & ~known)) return fail(ctx, VKGV_INVALID_ARG, "adjoint graph: unknown passes");
    const bool bwd = (passes & VKGV_DIFF_BACKWARD) != 0;
    DiffPlan D;
    int rc = diff_prepare(ctx, scene, views, view_count, bwd, scale, loss, grad_positions, grad_colors,
                          grad_texture, D);
    if (rc) return rc;
    vkgv_graph* g = new (std::nothrow) vkgv_graph();
    if (!g) return fail(ctx, VKGV_OUT_OF_MEMORY, "graph object");
    g->ctx = ctx;
    if (cudaMalloc(&g->d_views, sizeof(DeviceView) * view_count) != cudaSuccess ||
        cudaMemcpy(g->d_views, D.views.data(), sizeof(DeviceView) * view_count, cudaMemcpyHostToDevice) !=
            cudaSuccess) {
        cudaGetLastError();
        vkgv_graph_destroy(g);
        return fail(ctx, VKGV_OUT_OF_MEMORY, "graph view table");
    }
    cudaStream_t s = ctx->capture_stream;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaStreamBeginCapture");
    }
    if (passes & VKGV_DIFF_ZERO_GRADS) {
        const size_t nv = 3 * size_t(scene->vertex_count);
        const size_t nt = 3 * size_t(scene->tex_width) * scene->tex_height;
        if (loss) cudaMemsetAsync(reinterpret_cast<void*>(loss), 0, sizeof(float), s);
        if (grad_positions) cudaMemsetAsync(reinterpret_cast<void*>(grad_positions), 0, sizeof(float) * nv, s);
        if (grad_colors) cudaMemsetAsync(reinterpret_cast<void*>(grad_colors), 0, sizeof(float) * nv, s);
        if (grad_texture) cudaMemsetAsync(reinterpret_cast<void*>(grad_texture), 0, sizeof(float) * nt, s);
    }
    if (passes & VKGV_DIFF_FORWARD) diff_record(ctx, D, g->d_views, view_count, false, s);
    if (bwd) diff_record(ctx, D, g->d_views, view_count, true, s);
    e = cudaStreamEndCapture(s, &g->graph);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    *out_graph = g;
    return VKGV_OK;
}

int vkgv_graph_capture(vkgv_ctx* ctx, const vkgv_scene* scene, const vkgv_view* views, uint32_t view_count,
                       uint32_t flags, vkgv_graph** out_graph) {
    if (!ctx || !out_graph) return VKGV_INVALID_ARG;
    *out_graph = nullptr;
    if (!views || view_count == 0) return fail(ctx, VKGV_INVALID_ARG, "no views");
    int rc = two_pass_needs_pyramid(ctx, views, view_count, flags);
    if (rc) return rc;
    rc = ensure_views(ctx, view_count);
    if (rc) return rc;
    std::vector<DeviceView> host(view_count);
    Prepared P;
    rc = build_views(ctx, scene, views, view_count, flags, host.data(), P);
    if (rc) return rc;
    rc = attach_node_tables(ctx, P, host.data(), view_count, flags);
    if (rc) return rc;
    vkgv_graph* g = new (std::nothrow) vkgv_graph();
    if (!g) return fail(ctx, VKGV_OUT_OF_MEMORY, "graph object");
    g->ctx = ctx;
    if (cudaMalloc(&g->d_views, sizeof(DeviceView) * view_count) != cudaSuccess ||
        cudaMemcpy(g->d_views, host.data(), sizeof(DeviceView) * view_count, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        vkgv_graph_destroy(g);
        return fail(ctx, VKGV_OUT_OF_MEMORY, "graph view table");
    }
    cudaStream_t s = ctx->capture_stream;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaStreamBeginCapture");
    }
    record_frame(ctx, P, g->d_views, view_count, flags, s);
    e = cudaStreamEndCapture(s, &g->graph);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        vkgv_graph_destroy(g);
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    *out_graph = g;
    return VKGV_OK;
}

int vkgv_graph_launch(vkgv_graph* g, void* stream_) {
    if (!g || !g->exec) return VKGV_INVALID_ARG;
    cudaError_t e = cudaGraphLaunch(g->exec, reinterpret_cast<cudaStream_t>(stream_));
    if (e != cudaSuccess) return cuda_fail(g->ctx, e, "cudaGraphLaunch");
    return VKGV_OK;
}

int vkgv_graph_kernel_count(const vkgv_graph* g, uint32_t* out_count) {
    if (!g || !g->graph || !out_count) return VKGV_INVALID_ARG;
    size_t n = 0;
    if (cudaGraphGetNodes(g->graph, nullptr, &n) != cudaSuccess) return VKGV_CUDA_ERROR;
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g->graph, nodes.data(), &n) != cudaSuccess) return VKGV_CUDA_ERROR;
    uint32_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    *out_count = k;
    return VKGV_OK;
}

int vkgv_graph_destroy(vkgv_graph* g) {
    if (!g) return VKGV_INVALID_ARG;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->d_views) {
        cudaDeviceSynchronize();
        cudaFree(g->d_views);
    }
    delete g;
    return VKGV_OK;
}

int vkgv_autotune(const vkgv_config* base, const vkgv_scene* scene, const vkgv_view* views, uint32_t view_count,
                  uint32_t flags, uint32_t launches, vkgv_tune_entry* entries, uint32_t entry_capacity,
                  uint32_t* out_entry_count, vkgv_config* best) {
    if (!scene || !views || view_count == 0 || launches == 0 || !best) return VKGV_INVALID_ARG;
    static const uint32_t kBins[] = {8, 16, 32};
    static const uint32_t kSplits[] = {1, 2, 4};
    const vkgv_config b = base ? *base : vkgv_config{};
    if (b.device >= 0 && cudaSetDevice(b.device) != cudaSuccess) return VKGV_CUDA_ERROR;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (s) cudaStreamDestroy(s);
        if (e0) cudaEventDestroy(e0);
        return VKGV_CUDA_ERROR;
    }
    int rc = VKGV_OK;
    uint32_t n = 0;
    float best_ms = 0.f;
    for (uint32_t bin : kBins) {
        for (uint32_t split : kSplits) {
            vkgv_config c = b;
            c.bin_size = bin;
            c.meshlets_per_cta = split;
            vkgv_ctx* ctx = nullptr;
            vkgv_graph* g = nullptr;
            rc = vkgv_create(&c, &ctx);
            if (rc == VKGV_OK) rc = vkgv_graph_capture(ctx, scene, views, view_count, flags, &g);
            float ms = 0.f;
            if (rc == VKGV_OK) rc = vkgv_graph_launch(g, s);
            if (rc == VKGV_OK && cudaEventRecord(e0, s) != cudaSuccess) rc = VKGV_CUDA_ERROR;
            for (uint32_t i = 0; rc == VKGV_OK && i < launches; ++i) rc = vkgv_graph_launch(g, s);
            if (rc == VKGV_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                  cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                rc = VKGV_CUDA_ERROR;
            if (rc == VKGV_OK) {
                uint32_t code = 0, detail = 0;
                vkgv_device_status(ctx, &code, &detail);
                if (code) rc = VKGV_DEVICE_FAULT;
            }
            if (g) vkgv_graph_destroy(g);
            if (ctx) vkgv_destroy(ctx);
            if (rc != VKGV_OK) break;
            ms /= float(launches);
            if (entries && n < entry_capacity) entries[n] = vkgv_tune_entry{bin, split, ms, 0};
            ++n;
            if (n == 1 || ms < best_ms) {
                best_ms = ms;
                *best = c;
            }
        }
        if (rc != VKGV_OK) break;
    }
    cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (out_entry_count) *out_entry_count = std::min(n, entry_capacity);
    return rc;
}

}  // extern "C"
