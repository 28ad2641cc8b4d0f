// HiZ min-pyramid: the reduce chain of application.cpp:951-1003 running
// shaders/hiz_reduce.comp.glsl once per level.
//
// Level i (1..L) writes mip i-1 at size (W>>i, H>>i) from mip i-2 (the depth
// image for i = 1): texel p = MIN over the bilinear footprint of the source
// at ((p + 0.5) / size) with clamp-to-edge (the MIN-reduction sampler of
// application.cpp:437-458).  Where (W>>i, H>>i) has a zero dimension the
// reference dispatches no work and the mip stays undefined; it is defined
// here as 0.0 (far plane under reverse-Z, so it never occludes).  The
// reference's bounds test `pos > size` (hiz_reduce.comp.glsl:24) also lets
// pos == size through, whose image store is out of bounds; only pos < size is
// written here.
#include "kernels.cuh"

namespace vkgv {

namespace {

__device__ __forceinline__ float src_at(const unsigned long long* depth_id, const float* src, uint32_t sw,
                                        int x, int y) {
    if (depth_id) return u2f((uint32_t)(__ldg(depth_id + (size_t)y * sw + x) >> 32));
    return __ldg(src + (size_t)y * sw + x);
}

__global__ void __launch_bounds__(256) k_hiz_level(const DeviceView* __restrict__ views, uint32_t level) {
    const DeviceView& V = views[blockIdx.z];
    if (!V.pyr || level > V.pyr_levels) return;
    const uint32_t px = blockIdx.x * 32 + (threadIdx.x & 31);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 5);
    const uint32_t w0 = V.w >> 1, h0 = V.h >> 1;
    const uint32_t dw = V.w >> level, dh = V.h >> level;
    const uint32_t mw = mip_dim(w0, level - 1), mh = mip_dim(h0, level - 1);
    float* dst = V.pyr + mip_offset(w0, h0, level - 1);
    if (dw == 0 || dh == 0) {
        if (px < mw && py < mh) dst[(size_t)py * mw + px] = 0.0f;
        return;
    }
    if (px >= dw || py >= dh) return;
    const unsigned long long* depth_id = level == 1 ? V.depth_id : nullptr;
    const float* src = level == 1 ? nullptr : V.pyr + mip_offset(w0, h0, level - 2);
    const uint32_t sw = level == 1 ? V.w : mip_dim(w0, level - 2);
    const uint32_t sh = level == 1 ? V.h : mip_dim(h0, level - 2);
    const float u = fdiv(fadd((float)px, 0.5f), (float)dw);
    const float v = fdiv(fadd((float)py, 0.5f), (float)dh);
    int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
    const int nx = footprint_axis(u, sw, x0, x1);
    const int ny = footprint_axis(v, sh, y0, y1);
    float r = src_at(depth_id, src, sw, x0, y0);
    if (nx == 2) r = gmin(r, src_at(depth_id, src, sw, x1, y0));
    if (ny == 2) {
        r = gmin(r, src_at(depth_id, src, sw, x0, y1));
        if (nx == 2) r = gmin(r, src_at(depth_id, src, sw, x1, y1));
    }
    dst[(size_t)py * dw + px] = r;
}

}  // namespace

void launch_hiz(const DeviceView* views, uint32_t nviews, uint32_t max_w, uint32_t max_h, uint32_t sm_count,
                cudaStream_t stream) {
    (void)sm_count;
    uint32_t mx = max_w > max_h ? max_w : max_h, L = 0;
    while ((2u << L) <= mx) ++L;
    for (uint32_t i = 1; i <= L; ++i) {
        uint32_t w = mip_dim(max_w >> 1, i - 1), h = mip_dim(max_h >> 1, i - 1);
        dim3 grid((w + 31) / 32, (h + 7) / 8, nviews);
        k_hiz_level<<<grid, 256, 0, stream>>>(views, i);
    }
}

}  // namespace vkgv
