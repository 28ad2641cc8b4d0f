// Meshlet culling for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc at the point where they cull: a render
// loop that runs under CUDA stream capture in global mode (where cudaMalloc
// is not permitted), or an engine plugin whose host owns every device
// allocation and forbids the plugin to make its own.  vkgv_cull_static runs
// the same cull kernel as vkgv_cull without a context: its scratch (the
// view table, the per-view counters, the device status word and the list of
// pass-1 occlusion rejects that pass 2 re-tests) lives in one file-scope
// device array of fixed size, and the caller still passes the scene, the
// view and its survivor list.
//
// Limits and sharing:
//   - at most kStaticMaxDraws (262,144) meshlet draws; larger scenes are
//     rejected with VKGV_LIMIT_EXCEEDED;
//   - the array (about 1 MiB) is held by every GPU that loads the library
//     until the process exits;
//   - every call shares the array and leaves its contents for the next one
//     (pass 2 reads the rejects of the preceding pass-1 call); calls that
//     overlap on the GPU race with each other;
//   - the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress on that device, so make that first call before
//     any stream capture begins; the address is kept for the lifetime of the
//     device's primary context (a cudaDeviceReset ends it, so do not call
//     these entry points after one);
//   - device-side faults (a draw whose meshlet index is out of range, a
//     survivor list too short) go to the array's status words, which a pass-1
//     call clears; vkgv_cull_static_status reads and clears them.
#include <mutex>

#include "kernels.cuh"

namespace vkgv {
namespace {

constexpr uint32_t kStaticMaxDraws = 262144;

struct StaticScratch {
    DeviceView view;
    uint32_t counters[4];
    uint32_t status[2];
    uint32_t _pad[2];
    uint32_t rejected[kStaticMaxDraws];
};

// The scratch: one file-scope device array, 256-byte aligned.
static __device__ __align__(256) unsigned char g_cull_scratch[(sizeof(StaticScratch) + 255) / 256 * 256];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
uint32_t g_sm_count[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Resolves the array's device address once per device (that device
// current), since the host-side symbol is not a device address.
int scratch_for_current_device(StaticScratch** out, uint32_t* sm_count) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VKGV_CUDA_ERROR;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_cull_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return VKGV_CUDA_ERROR;
        }
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return VKGV_CUDA_ERROR;
        g_scratch_addr[dev] = p;
        g_sm_count[dev] = (uint32_t)(sms > 0 ? sms : 1);
    }
    *out = static_cast<StaticScratch*>(g_scratch_addr[dev]);
    *sm_count = g_sm_count[dev];
    return VKGV_OK;
}

// Writes the view table entry and clears what this pass must start from
// zero: pass 1 clears every counter and the status word; pass 2 keeps the
// pass-1 survivor and reject counts and clears its own survivor count.
__global__ void k_stage_static_view(DeviceView v, StaticScratch* s, uint32_t pass) {
    if (threadIdx.x == 0) s->view = v;
    if (pass == 1) {
        if (threadIdx.x < 4) s->counters[threadIdx.x] = 0;
        if (threadIdx.x < 2) s->status[threadIdx.x] = 0;
    } else if (threadIdx.x == 2) {
        s->counters[2] = 0;
    }
}

}  // namespace
}  // namespace vkgv

using namespace vkgv;

extern "C" int vkgv_cull_static(const vkgv_scene* scene, const vkgv_view* view, uint32_t flags, uint32_t pass,
                                void* stream_) {
    if (!scene || !view) return VKGV_INVALID_ARG;
    if (pass != 1 && pass != 2) return VKGV_INVALID_ARG;
    const uint32_t D = scene->meshlet_draw_count;
    if (D > kStaticMaxDraws) return VKGV_LIMIT_EXCEEDED;
    if (D > 0 && (!scene->draw_buffer || !scene->transform_buffer || !scene->primitive_buffer ||
                  !scene->material_buffer))
        return VKGV_INVALID_ARG;
    if (view->width == 0 || view->height == 0 || !view->camera_buffer) return VKGV_INVALID_ARG;
    if (view->width > VKGV_MAX_VIEW_DIM || view->height > VKGV_MAX_VIEW_DIM) return VKGV_LIMIT_EXCEEDED;
    if (!view->survivors || !view->survivor_count || view->survivor_capacity < D) return VKGV_INVALID_ARG;
    uint32_t levels = 0;
    uint64_t floats = 0;
    if (vkgv_pyramid_layout(view->width, view->height, &levels, &floats) != VKGV_OK) return VKGV_INVALID_ARG;
    const vkgv_pyramid* pyrs[2] = {&view->prev_pyramid, &view->pyramid};
    for (const vkgv_pyramid* p : pyrs)
        if (p->levels && (!p->data || p->width != (view->width >> 1) || p->height != (view->height >> 1) ||
                          p->levels != levels || (p->data & 3u)))
            return VKGV_INVALID_ARG;

    StaticScratch* s = nullptr;
    uint32_t sm_count = 1;
    int rc = scratch_for_current_device(&s, &sm_count);
    if (rc != VKGV_OK) return rc;

    SceneArgs S;
    S.draws = reinterpret_cast<const vkgv_meshlet_draw*>(scene->draw_buffer);
    S.transforms = reinterpret_cast<const float*>(scene->transform_buffer);
    S.prims = reinterpret_cast<const vkgv_primitive*>(scene->primitive_buffer);
    S.mats = reinterpret_cast<const vkgv_material*>(scene->material_buffer);
    S.textures = reinterpret_cast<const vkgv_texture*>(scene->texture_table);
    S.draw_count = D;
    S.texture_count = scene->texture_count;
    S.cone_table = reinterpret_cast<const uint64_t*>(scene->cone_table);
    S.primitive_count = scene->cone_table ? scene->primitive_count : 0;
    S.transform_count = scene->transform_count;
    S.tdets = nullptr;

    DeviceView v{};
    v.cam = reinterpret_cast<const vkgv_camera*>(view->camera_buffer);
    v.w = view->width;
    v.h = view->height;
    v.prev_pyr = reinterpret_cast<const float*>(view->prev_pyramid.data);
    v.prev_w0 = view->prev_pyramid.width;
    v.prev_h0 = view->prev_pyramid.height;
    v.prev_levels = view->prev_pyramid.levels;
    v.pyr = reinterpret_cast<float*>(view->pyramid.data);
    v.pyr_levels = view->pyramid.levels;
    v.depth_id = reinterpret_cast<unsigned long long*>(view->depth_id);
    v.survivors = reinterpret_cast<uint32_t*>(view->survivors);
    v.survivor_count = reinterpret_cast<uint32_t*>(view->survivor_count);
    v.survivor_capacity = view->survivor_capacity;
    v.rejected = s->rejected;
    v.counters = s->counters;

    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    k_stage_static_view<<<1, 32, 0, stream>>>(v, s, pass);
    launch_cull(S, &s->view, 1, flags, pass, s->status, sm_count, stream);
    launch_finalize(&s->view, 1, stream);
    if (cudaGetLastError() != cudaSuccess) return VKGV_CUDA_ERROR;
    return VKGV_OK;
}

extern "C" int vkgv_cull_static_status(void* stream_, uint32_t* out_code, uint32_t* out_detail) {
    if (!out_code || !out_detail) return VKGV_INVALID_ARG;
    StaticScratch* s = nullptr;
    uint32_t sm_count = 1;
    int rc = scratch_for_current_device(&s, &sm_count);
    if (rc != VKGV_OK) return rc;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    uint32_t words[2] = {0u, 0u};
    // stream-ordered after the culls on `stream`; the words then start again
    // from zero for the calls that follow
    if (cudaMemcpyAsync(words, s->status, sizeof(words), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess ||
        cudaMemsetAsync(s->status, 0, sizeof(words), stream) != cudaSuccess) {
        cudaGetLastError();
        return VKGV_CUDA_ERROR;
    }
    *out_code = words[0];
    *out_detail = words[1];
    return VKGV_OK;
}
