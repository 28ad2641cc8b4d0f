// Visibility-buffer resolve (shaders/visbuffer/visbuffer_resolve.comp.glsl:17-41)
// plus the per-frame clear and the survivor-count finalisation.
//
// Flat resolve: per pixel, unpack the ID, fetch draw -> primitive ->
// material and store fromLinear(albedoFactor) (shaders/srgb.h.glsl:26-32) as
// RGBA8 UNORM, or 0 where nothing was drawn.  The reference dispatches
// floor(W/32) x H groups (application.cpp:945), leaving the last W mod 32
// columns unwritten; every column is written here.
//
// Textured resolve (extension, no reference implementation): the commented-out
// formula of visbuffer.frag.glsl:29-34 — perspective-correct barycentrics of
// the visible triangle, vertex colour, transformUv (mesh_common.h.glsl:129-135)
// and a bilinear REPEAT base-colour sample decoded with toLinear.
#include <cuda_fp16.h>

#include "kernels.cuh"

namespace vkgv {

namespace {

// fromLinear / toLinear (shaders/srgb.h.glsl:9-23), with the operation
// order of the oracle so that only powf's last ulp can differ.
__device__ __forceinline__ float from_linear(float c) {
    const bool cutoff = c < 0.0031308f;
    const float higher = fsub(fmul(1.055f, powf(c, 1.0f / 2.4f)), 0.055f);
    const float lower = fmul(c, 12.92f);
    return cutoff ? lower : higher;
}

__device__ __forceinline__ float to_linear(float c) {
    const bool cutoff = c < 0.04045f;
    const float higher = powf(fdiv(fadd(c, 0.055f), 1.055f), 2.4f);
    const float lower = fdiv(c, 12.92f);
    return cutoff ? lower : higher;
}

// The textured resolve is compared within 1/255; its sRGB curves use the
// hardware exp2/log2 pow (relative error ~1e-6, which can move a channel by
// one step only at a rounding boundary) and multiply by the reciprocals of
// 1.055 and 12.92 (one ulp from the quotients) on the filtered colour.
__device__ __forceinline__ float from_linear_fast(float c) {
    const bool cutoff = c < 0.0031308f;
    const float higher = fsub(fmul(1.055f, __powf(c, 1.0f / 2.4f)), 0.055f);
    const float lower = fmul(c, 12.92f);
    return cutoff ? lower : higher;
}

__device__ __forceinline__ float to_linear_fast(float c) {
    const bool cutoff = c < 0.04045f;
    const float higher = __powf(fmul(fadd(c, 0.055f), 1.0f / 1.055f), 2.4f);
    const float lower = fmul(c, 1.0f / 12.92f);
    return cutoff ? lower : higher;
}

__device__ __forceinline__ uint32_t unorm8(float c) {
    if (!(c > 0.0f)) return 0;
    if (c > 1.0f) c = 1.0f;
    return (uint32_t)__float2int_rn(fmul(c, 255.0f));
}

__device__ __forceinline__ uint32_t pack_rgba(const float lin[4]) {
    return unorm8(from_linear(lin[0])) | (unorm8(from_linear(lin[1])) << 8) | (unorm8(from_linear(lin[2])) << 16) |
           (unorm8(lin[3]) << 24);
}

__device__ __forceinline__ uint32_t pack_rgba_fast(const float lin[4]) {
    return unorm8(from_linear_fast(lin[0])) | (unorm8(from_linear_fast(lin[1])) << 8) |
           (unorm8(from_linear_fast(lin[2])) << 16) | (unorm8(lin[3]) << 24);
}

__device__ __forceinline__ float lerp(float a, float b, float t) { return fadd(a, fmul(t, fsub(b, a))); }

// Total survivors of the frame (pass 1 + pass 2) into the caller's counter.
__device__ __forceinline__ void finalize_view(const DeviceView& V) {
    if (!V.survivor_count) return;
    const uint32_t c0 = min(V.counters[0], V.survivor_capacity);
    const uint32_t c2 = min(V.counters[2], V.survivor_capacity - c0);
    *V.survivor_count = c0 + c2;
}

// REPEAT addressing: the non-negative remainder of i by n (n >= 1), with a
// mask for power-of-two sizes and 32-bit arithmetic where i fits.
__device__ __forceinline__ uint32_t wrap_texel(long long i, uint32_t n) {
    if ((n & (n - 1)) == 0) return (uint32_t)(i & (long long)(n - 1));
    if (i >= 0 && i < 0x7fffffffll) return (uint32_t)i % n;
    const long long r = i % (long long)n;
    return (uint32_t)(r < 0 ? r + n : r);
}

// Bilinear REPEAT sample, texel centres at +0.5.  Textured shading of a
// high-frequency texture is very sensitive to the sample position, so every
// operation follows the oracle's order (no contraction).
__device__ void sample_texture(const vkgv_texture& t, float u, float v, const float* unorm, float out[4]) {
    const float tx = fsub(fmul(u, (float)t.width), 0.5f), ty = fsub(fmul(v, (float)t.height), 0.5f);
    const float fx = floorf(tx), fy = floorf(ty);
    const float ax = fsub(tx, fx), ay = fsub(ty, fy);
    const long long x0 = (long long)fx, y0 = (long long)fy;
    const uint32_t xs[2] = {wrap_texel(x0, t.width), wrap_texel(x0 + 1, t.width)};
    const uint32_t ys[2] = {wrap_texel(y0, t.height), wrap_texel(y0 + 1, t.height)};
    float tex[2][2][4];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const size_t idx = (size_t)ys[j] * t.row_pitch + (size_t)xs[i];
            if (t.format == VKGV_TEXTURE_RGBA8) {
                const uchar4 p = __ldg(reinterpret_cast<const uchar4*>(t.data) + idx);
                tex[j][i][0] = unorm[p.x];
                tex[j][i][1] = unorm[p.y];
                tex[j][i][2] = unorm[p.z];
                tex[j][i][3] = unorm[p.w];
            } else {
                const float* p = reinterpret_cast<const float*>(t.data) + 3 * idx;
                tex[j][i][0] = __ldg(p);
                tex[j][i][1] = __ldg(p + 1);
                tex[j][i][2] = __ldg(p + 2);
                tex[j][i][3] = 1.0f;
            }
        }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float top = lerp(tex[0][0][k], tex[0][1][k], ax);
        const float bot = lerp(tex[1][0][k], tex[1][1][k], ax);
        out[k] = lerp(top, bot, ay);
    }
}

// The visible fragment of one pixel: its triangle's three vertices in clip
// space and the perspective-correct barycentrics of the pixel centre.
struct Frag {
    const vkgv_vertex* vx[3];
    const vkgv_material* mat;
    uint32_t transform_index;
    uint32_t color[3];  // the vertices' RGBA8 (textured resolve only)
    uint32_t uv[3];     // the vertices' two binary16 UVs, u in the low half (textured resolve only)
    float l[3];
    float pos[3];  // the interpolated clip position x, y, w (motion vectors only)
};

// A 24-byte vertex record read as three 8-byte words: (x, y), (z, colour),
// (normal + pad, uv).  Vertex buffers are 8-byte aligned (the raster reads
// positions as float2 too).
__device__ __forceinline__ void load_vertex(const vkgv_vertex* v, bool full, float& x, float& y, float& z,
                                            uint32_t& color, uint32_t& uv) {
    const uint2* r = reinterpret_cast<const uint2*>(v);
    const uint2 a = __ldg(r), b = __ldg(r + 1);
    x = __uint_as_float(a.x);
    y = __uint_as_float(a.y);
    z = __uint_as_float(b.x);
    color = b.y;
    uv = full ? __ldg(r + 2).y : 0u;
}

// Loads a 4x4 node-table matrix (16-byte aligned rows of the table).
__device__ __forceinline__ void load_m4(const float* src, float m[16]) {
    const float4* q = reinterpret_cast<const float4*>(src);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float4 c = __ldg(q + k);
        m[4 * k] = c.x, m[4 * k + 1] = c.y, m[4 * k + 2] = c.z, m[4 * k + 3] = c.w;
    }
}

// vp * transforms[node] without a node table (the stage entry points); kept
// out of line so that its registers do not weigh on the table path.
__device__ __noinline__ void direct_mvp(const float* __restrict__ transforms, const float* vp, uint32_t node,
                                        float mvp[16]) {
    const float* Mp = transforms + 16 * (size_t)node;
    float M[16], VP[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        M[k] = __ldg(Mp + k);
        VP[k] = vp[k];
    }
    m4m(VP, M, mvp);
}

// vp * transforms[node], from the per-view node table when the frame has one.
// The out-of-line product writes a separate array, so that `mvp` itself
// stays in registers on the table path.
__device__ __forceinline__ void node_mvp(const SceneArgs& S, const float* table, const float* vp, uint32_t node,
                                         float mvp[16]) {
    if (table && node < S.transform_count) {
        load_m4(table + 16 * (size_t)node, mvp);
    } else {
        float fb[16];
        direct_mvp(S.transforms, vp, node, fb);
#pragma unroll
        for (int k = 0; k < 16; ++k) mvp[k] = fb[k];
    }
}

__device__ __forceinline__ float interp3(const float l[3], float v0, float v1, float v2) {
    return fadd(fadd(fmul(l[0], v0), fmul(l[1], v1)), fmul(l[2], v2));
}

template <bool MOTION, bool TEXTURED>
__device__ void frag_setup(const SceneArgs& S, const DeviceView& V, uint32_t px, uint32_t py, uint32_t id, Frag& f) {
    const uint32_t d = id >> VKGV_TRIANGLE_BITS, t = id & ((1u << VKGV_TRIANGLE_BITS) - 1u);
    const vkgv_meshlet_draw dr = S.draws[d];
    const vkgv_primitive* prim = &S.prims[dr.primitive_index];
    const vkgv_meshlet* ml = reinterpret_cast<const vkgv_meshlet*>(prim->meshlet_buffer) + dr.meshlet_index;
    f.mat = &S.mats[prim->material_index];
    f.transform_index = dr.transform_index;
    float mvp[16];
    node_mvp(S, V.mvps, V.cam->view_projection, dr.transform_index, mvp);
    const uint8_t* tri = reinterpret_cast<const uint8_t*>(prim->primitive_index_buffer) + ml->triangle_offset + 3 * t;
    const uint32_t* vidx = reinterpret_cast<const uint32_t*>(prim->vertex_index_buffer) + ml->vertex_offset;
    const vkgv_vertex* verts = reinterpret_cast<const vkgv_vertex*>(prim->vertex_buffer);
    float c[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f.vx[k] = verts + vidx[tri[k]];
        float x, y, z;
        load_vertex(f.vx[k], TEXTURED, x, y, z, f.color[k], f.uv[k]);
        m4v(mvp, x, y, z, 1.0f, c[k]);
    }
    // Perspective-correct barycentrics: the clip-space weights whose point
    // projects to the pixel centre are proportional to a x b.
    const float nx = fsub(fmul(fdiv(fadd((float)px, 0.5f), (float)V.w), 2.0f), 1.0f);
    const float ny = fsub(fmul(fdiv(fadd((float)py, 0.5f), (float)V.h), 2.0f), 1.0f);
    float a[3], b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = fsub(c[k][0], fmul(nx, c[k][3]));
        b[k] = fsub(c[k][1], fmul(ny, c[k][3]));
    }
    f.l[0] = fsub(fmul(a[1], b[2]), fmul(a[2], b[1]));
    f.l[1] = fsub(fmul(a[2], b[0]), fmul(a[0], b[2]));
    f.l[2] = fsub(fmul(a[0], b[1]), fmul(a[1], b[0]));
    const float sum = fadd(fadd(f.l[0], f.l[1]), f.l[2]);
    if (sum != 0.0f) {
        f.l[0] = fdiv(f.l[0], sum);
        f.l[1] = fdiv(f.l[1], sum);
        f.l[2] = fdiv(f.l[2], sum);
    } else {
        f.l[0] = f.l[1] = f.l[2] = 1.0f / 3.0f;
    }
    if (MOTION) {
        f.pos[0] = interp3(f.l, c[0][0], c[1][0], c[2][0]);
        f.pos[1] = interp3(f.l, c[0][1], c[1][1], c[2][1]);
        f.pos[2] = interp3(f.l, c[0][3], c[1][3], c[2][3]);
    }
}

// unorm[i] = i / 255 (correctly rounded), a per-block table in shared memory.
__device__ void shade_textured(const SceneArgs& S, const Frag& f, const float* unorm, float out[4]) {
    const vkgv_material& mat = *f.mat;
    float col[4], uv[2];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        col[k] = interp3(f.l, unorm[(f.color[0] >> (8 * k)) & 255u], unorm[(f.color[1] >> (8 * k)) & 255u],
                         unorm[(f.color[2] >> (8 * k)) & 255u]);
#pragma unroll
    for (int k = 0; k < 2; ++k)
        uv[k] = interp3(f.l, __half2float(__ushort_as_half((unsigned short)(f.uv[0] >> (16 * k)))),
                        __half2float(__ushort_as_half((unsigned short)(f.uv[1] >> (16 * k)))),
                        __half2float(__ushort_as_half((unsigned short)(f.uv[2] >> (16 * k)))));
    float sampled[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    if (mat.albedo_index != VKGV_INVALID_HANDLE && mat.albedo_index < S.texture_count) {
        // transformUv (mesh_common.h.glsl:129-135): rotate, scale, offset
        // sincos(+-0) = (+-0, 1) exactly; skip the reduction for unrotated UVs
        float sn = mat.uv_rotation, cs = 1.0f;
        if (mat.uv_rotation != 0.0f) sincosf(mat.uv_rotation, &sn, &cs);
        const float ru = fadd(fmul(cs, uv[0]), fmul(sn, uv[1]));
        const float rv = fadd(fmul(-sn, uv[0]), fmul(cs, uv[1]));
        const float tu = fadd(fmul(ru, mat.uv_scale[0]), mat.uv_offset[0]);
        const float tv = fadd(fmul(rv, mat.uv_scale[1]), mat.uv_offset[1]);
        const vkgv_texture tex = S.textures[mat.albedo_index];
        sample_texture(tex, tu, tv, unorm, sampled);
        if (tex.format == VKGV_TEXTURE_RGBA8)
#pragma unroll
            for (int k = 0; k < 3; ++k) sampled[k] = to_linear_fast(sampled[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = fmul(fmul(col[k], mat.albedo_factor[k]), sampled[k]);
}

// Motion vector of the visible fragment (visbuffer.frag.glsl:38, with the
// mesh shader's position / prevPosition varyings of visbuffer.mesh.glsl:44-64):
//   position     = viewProjection     * M * vertex, interpolated
//   prevPosition = prevViewProjection * M * vertex, interpolated
//   motion = (prev.xy / prev.w * 0.5 - 0.5) - (pos.xy / pos.w * 0.5 - 0.5)
// M is the node's current transform for both (the reference has no
// previous-frame transforms).  Written as two RN binary16, x in the low half.
// Only the x, y and w rows of prevViewProjection * M are needed; each
// vertex's previous clip position is folded into the interpolation sums
// ((l0 p0 + l1 p1) + l2 p2) as it is computed, which keeps the variant small
// enough for six CTAs per SM.
__device__ uint32_t motion_vector(const SceneArgs& S, const DeviceView& V, const Frag& f) {
    float rx[4], ry[4], rw[4];  // rows x, y, w of prev_view_projection * M (per column)
    if (V.prev_mvps && f.transform_index < S.transform_count) {
        const float4* q = reinterpret_cast<const float4*>(V.prev_mvps + 16 * (size_t)f.transform_index);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float4 col = __ldg(q + c);
            rx[c] = col.x, ry[c] = col.y, rw[c] = col.w;
        }
    } else {
        float pm[16];
        node_mvp(S, nullptr, V.cam->prev_view_projection, f.transform_index, pm);
#pragma unroll
        for (int c = 0; c < 4; ++c) rx[c] = pm[4 * c], ry[c] = pm[4 * c + 1], rw[c] = pm[4 * c + 3];
    }
    float px = 0.0f, py = 0.0f, pw = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 xy = __ldg(reinterpret_cast<const float2*>(f.vx[k]->position));
        const float x = xy.x, y = xy.y, z = __ldg(&f.vx[k]->position[2]);
        // m4v's order: ((m0 x + m1 y) + m2 z) + m3
        const float cx = fadd(fadd(fadd(fmul(rx[0], x), fmul(rx[1], y)), fmul(rx[2], z)), fmul(rx[3], 1.0f));
        const float cy = fadd(fadd(fadd(fmul(ry[0], x), fmul(ry[1], y)), fmul(ry[2], z)), fmul(ry[3], 1.0f));
        const float cw = fadd(fadd(fadd(fmul(rw[0], x), fmul(rw[1], y)), fmul(rw[2], z)), fmul(rw[3], 1.0f));
        if (k == 0) {
            px = fmul(f.l[0], cx), py = fmul(f.l[0], cy), pw = fmul(f.l[0], cw);
        } else {
            px = fadd(px, fmul(f.l[k], cx)), py = fadd(py, fmul(f.l[k], cy)), pw = fadd(pw, fmul(f.l[k], cw));
        }
    }
    const float cur_x = fsub(fmul(fdiv(f.pos[0], f.pos[2]), 0.5f), 0.5f);
    const float cur_y = fsub(fmul(fdiv(f.pos[1], f.pos[2]), 0.5f), 0.5f);
    const float prev_x = fsub(fmul(fdiv(px, pw), 0.5f), 0.5f);
    const float prev_y = fsub(fmul(fdiv(py, pw), 0.5f), 0.5f);
    return (uint32_t)__half_as_ushort(__float2half_rn(fsub(prev_x, cur_x))) |
           ((uint32_t)__half_as_ushort(__float2half_rn(fsub(prev_y, cur_y))) << 16);
}

// One pixel of the resolve: its id, and its colour and motion vector.
// The outputs a resolve writes for one view (null where the flags skip them).
struct ResolveOut {
    uint32_t* ids;
    uint32_t* rgba;
    uint32_t* motion;
};

template <bool MOTION>
__device__ __forceinline__ ResolveOut resolve_outputs(const DeviceView& V, uint32_t flags) {
    return {(flags & VKGV_WRITE_IDS) ? V.ids : nullptr,
            (flags & (VKGV_RESOLVE_FLAT | VKGV_RESOLVE_TEXTURED)) ? V.rgba : nullptr, MOTION ? V.motion : nullptr};
}

template <bool TEXTURED, bool MOTION>
__device__ __forceinline__ void resolve_pixel(const SceneArgs& S, const DeviceView& V, const float* s_unorm,
                                              const ResolveOut& o, uint32_t w, uint32_t p) {
    uint32_t* ids = o.ids;
    uint32_t* rgba = o.rgba;
    uint32_t* motion = o.motion;
    const uint32_t lo = (uint32_t)__ldcs(V.depth_id + p);
    const uint32_t id = lo ? lo - 1u : VKGV_VISBUFFER_CLEAR;
    if (ids) __stcs(ids + p, id);
    if (!rgba && !MOTION) return;
    uint32_t out = 0, mv = 0;
    if (id != VKGV_VISBUFFER_CLEAR) {
        float lin[4];
        if (TEXTURED || MOTION) {
            Frag f;
            frag_setup<MOTION, TEXTURED>(S, V, p % w, p / w, id, f);
            if (MOTION) mv = motion_vector(S, V, f);
            if (TEXTURED) {
                shade_textured(S, f, s_unorm, lin);
            } else {
                const float4 a = *reinterpret_cast<const float4*>(f.mat->albedo_factor);
                lin[0] = a.x, lin[1] = a.y, lin[2] = a.z, lin[3] = a.w;
            }
        } else {
            const vkgv_meshlet_draw dr = S.draws[id >> VKGV_TRIANGLE_BITS];
            const vkgv_material& mat = S.mats[S.prims[dr.primitive_index].material_index];
            const float4 a = *reinterpret_cast<const float4*>(mat.albedo_factor);
            lin[0] = a.x, lin[1] = a.y, lin[2] = a.z, lin[3] = a.w;
        }
        if (rgba) out = TEXTURED ? pack_rgba_fast(lin) : pack_rgba(lin);
    }
    if (rgba) __stcs(rgba + p, out);
    if (MOTION) __stcs(motion + p, mv);
}

template <bool TEXTURED, bool MOTION>
__global__ void __launch_bounds__(256, 6) k_resolve(SceneArgs S, const DeviceView* __restrict__ views, uint32_t flags) {
    pdl_begin();
    const DeviceView& V = views[blockIdx.y];
    __shared__ float s_unorm[256];
    if (TEXTURED) {
        s_unorm[threadIdx.x] = fdiv((float)threadIdx.x, 255.0f);  // blockDim.x == 256
        __syncthreads();
    }
    const uint32_t w = V.w, n = V.w * V.h;
    const ResolveOut o = resolve_outputs<MOTION>(V, flags);
    if (blockIdx.x == 0 && threadIdx.x == 0) finalize_view(V);
    // two pixels per thread (the launch sizes the grid for it), so that the
    // compiler interleaves their load chains: 1080p textured 59.4 -> 57.3 us
#pragma unroll 2
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        resolve_pixel<TEXTURED, MOTION>(S, V, s_unorm, o, w, p);
}

// Several views: one wave of resident CTAs whose warps take chunks of
// kResolveChunk pixels (all views' chunks numbered in view order) from a
// global counter, so views smaller than the largest cost no empty CTAs.
// A chunk is 64 tiles of 8 x 4 pixels (row-major over the view, one tile per
// warp step): the pixels of a warp share more triangles and texels than a
// 32-pixel row (256-view batch: 4.13 -> 3.89 ms).  The warp that takes a
// view's first chunk finalizes the view; the last CTA to finish returns the
// counters to zero.
constexpr uint32_t kResolveChunk = 2048;
constexpr uint32_t kResolveMaxViews = 4096;
constexpr uint32_t kTileW = 8, kTileH = 4;  // kTileW * kTileH == 32

// Tiled pixel slots of a view: whole 8 x 4 tiles, padded past its edges.
__device__ __forceinline__ uint32_t tile_slots(uint32_t w, uint32_t h) {
    return ((w + kTileW - 1) / kTileW) * ((h + kTileH - 1) / kTileH) * 32u;
}

template <bool TEXTURED, bool MOTION>
__global__ void __launch_bounds__(256, 6) k_resolve_chunks(SceneArgs S, const DeviceView* __restrict__ views,
                                                           uint32_t nviews, uint32_t flags, uint32_t* work) {
    pdl_begin();
    __shared__ float s_unorm[256];
    __shared__ uint32_t s_pre[kResolveMaxViews + 1];
    if (TEXTURED) s_unorm[threadIdx.x] = fdiv((float)threadIdx.x, 255.0f);  // blockDim.x == 256
    for (uint32_t v = threadIdx.x; v < nviews; v += blockDim.x)
        s_pre[v + 1] = (tile_slots(views[v].w, views[v].h) + kResolveChunk - 1) / kResolveChunk;
    if (threadIdx.x == 0) s_pre[0] = 0;
    __syncthreads();
    if (threadIdx.x < 32) {
        // inclusive scan of s_pre[1..nviews]: lane-contiguous segments, then
        // a warp scan of the segment sums
        const uint32_t lane = threadIdx.x, seg = (nviews + 31) / 32;
        const uint32_t b = 1 + lane * seg, e = min(b + seg, nviews + 1);
        uint32_t sum = 0;
        for (uint32_t i = b; i < e; ++i) sum += s_pre[i];
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        uint32_t run = incl - sum;
        for (uint32_t i = b; i < e; ++i) {
            run += s_pre[i];
            s_pre[i] = run;
        }
    }
    __syncthreads();
    const uint32_t total = s_pre[nviews];
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        uint32_t v = 0, hi = nviews;
        while (v + 1 < hi) {
            const uint32_t mid = (v + hi) >> 1;
            if (s_pre[mid] <= item) v = mid;
            else hi = mid;
        }
        const DeviceView& V = views[v];
        if (item == s_pre[v] && lane == 0) finalize_view(V);
        const uint32_t w = V.w, h = V.h, base = (item - s_pre[v]) * kResolveChunk;
        const uint32_t tiles_per_row = (w + kTileW - 1) / kTileW;
        const ResolveOut o = resolve_outputs<MOTION>(V, flags);
#pragma unroll 1
        for (uint32_t j = lane; j < kResolveChunk; j += 32) {
            const uint32_t t = (base + j) >> 5;
            const uint32_t x = (t % tiles_per_row) * kTileW + lane % kTileW;
            const uint32_t y = (t / tiles_per_row) * kTileH + lane / kTileW;
            if (x < w && y < h) resolve_pixel<TEXTURED, MOTION>(S, V, s_unorm, o, w, y * w + x);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(work + 1, 1u) == gridDim.x - 1) {
            work[0] = 0;
            work[1] = 0;
        }
    }
}

__global__ void __launch_bounds__(256) k_clear(const DeviceView* __restrict__ views, uint32_t* counters,
                                               uint32_t counter_words, uint32_t skip_pixels,
                                               const float* __restrict__ transforms, uint32_t transform_count,
                                               float* __restrict__ tdets) {
    pdl_begin();
    const DeviceView& V = views[blockIdx.y];
    if (transform_count) {
        // the view's node tables: view_projection * M, for motion-vector
        // frames prev_view_projection * M, and for cone-culled frames the
        // raster eye in each node's object space
        __shared__ float s_vp[2][16];
        __shared__ float s_eye[3];
        __shared__ int s_eye_ok;
        if (threadIdx.x < 16) s_vp[0][threadIdx.x] = V.cam->view_projection[threadIdx.x];
        if (threadIdx.x >= 32 && threadIdx.x < 48)
            s_vp[1][threadIdx.x - 32] = V.cam->prev_view_projection[threadIdx.x - 32];
        if (threadIdx.x == 64 && V.eyes) {
            float vp[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) vp[k] = V.cam->view_projection[k];
            s_eye_ok = eye_from_vp(vp, s_eye);
        }
        __syncthreads();
        float* out = const_cast<float*>(V.mvps);
        float* prev = const_cast<float*>(V.prev_mvps);
        float4* eyes = const_cast<float4*>(V.eyes);
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < transform_count; i += gridDim.x * blockDim.x) {
            float M[16], r[16];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 q = __ldg(reinterpret_cast<const float4*>(transforms + 16 * (size_t)i) + k);
                M[4 * k] = q.x, M[4 * k + 1] = q.y, M[4 * k + 2] = q.z, M[4 * k + 3] = q.w;
            }
            if (blockIdx.y == 0) tdets[i] = det4(M);
            m4m(s_vp[0], M, r);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                reinterpret_cast<float4*>(out + 16 * (size_t)i)[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2],
                                                                                  r[4 * k + 3]);
            if (eyes) {
                float o[3] = {0.0f, 0.0f, 0.0f};
                const bool ok = s_eye_ok && object_eye(M, s_eye, o);
                eyes[i] = make_float4(o[0], o[1], o[2], ok ? 1.0f : 0.0f);
            }
            if (prev) {
                m4m(s_vp[1], M, r);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    reinterpret_cast<float4*>(prev + 16 * (size_t)i)[k] =
                        make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
            }
        }
    }
    if (counters) {
        if (blockIdx.x == 0 && threadIdx.x < 8) V.counters[threadIdx.x] = 0;
        if (blockIdx.x == 0 && blockIdx.y == 0)
            for (uint32_t i = threadIdx.x; i < counter_words; i += blockDim.x) counters[i] = 0;
    }
    if (skip_pixels) return;
    const uint32_t n = V.w * V.h;
    // 16-byte stores of two pixels; depth_id allocations are 16-byte aligned
    // when they come from cudaMalloc (checked by the host).
    ulonglong2* p2 = reinterpret_cast<ulonglong2*>(V.depth_id);
    const uint32_t n2 = n / 2;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x)
        __stcg(p2 + i, make_ulonglong2(0ull, 0ull));
    if ((n & 1u) && blockIdx.x == 0 && threadIdx.x == 0) V.depth_id[n - 1] = 0ull;
}

__global__ void k_finalize(const DeviceView* __restrict__ views, uint32_t nviews) {
    pdl_begin();
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nviews) return;
    finalize_view(views[v]);
}

}  // namespace

template <bool T, bool M>
bool launch_resolve_chunks(const SceneArgs& S, const DeviceView* views, uint32_t nviews, uint32_t flags,
                           uint32_t* work, uint32_t sm_count, cudaStream_t stream) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resolve_chunks<T, M>, 256, 0) != cudaSuccess ||
        per_sm <= 0) {
        cudaGetLastError();
        return false;
    }
    launch_pdl(k_resolve_chunks<T, M>, dim3(sm_count * (uint32_t)per_sm), dim3(256), 0, stream, S, views, nviews,
               flags, work);
    return true;
}

void launch_resolve(const SceneArgs& S, const DeviceView* views, uint32_t nviews, uint32_t max_w, uint32_t max_h,
                    uint32_t flags, uint32_t* work, uint32_t sm_count, cudaStream_t stream) {
    const bool tex = (flags & VKGV_RESOLVE_TEXTURED) != 0, mv = (flags & VKGV_WRITE_MOTION) != 0;
    if (nviews > 1 && nviews <= kResolveMaxViews && work && sm_count) {
        const bool done = tex && mv ? launch_resolve_chunks<true, true>(S, views, nviews, flags, work, sm_count, stream)
                          : tex     ? launch_resolve_chunks<true, false>(S, views, nviews, flags, work, sm_count, stream)
                          : mv      ? launch_resolve_chunks<false, true>(S, views, nviews, flags, work, sm_count, stream)
                                    : launch_resolve_chunks<false, false>(S, views, nviews, flags, work, sm_count, stream);
        if (done) return;
    }
    const uint64_t px = (uint64_t)max_w * max_h;
    uint32_t bx = (uint32_t)((px + 511) / 512);
    if (bx > 65535u) bx = 65535u;
    dim3 grid(bx, nviews);
    if (tex && mv)
        launch_pdl(k_resolve<true, true>, grid, dim3(256), 0, stream, S, views, flags);
    else if (tex)
        launch_pdl(k_resolve<true, false>, grid, dim3(256), 0, stream, S, views, flags);
    else if (mv)
        launch_pdl(k_resolve<false, true>, grid, dim3(256), 0, stream, S, views, flags);
    else
        launch_pdl(k_resolve<false, false>, grid, dim3(256), 0, stream, S, views, flags);
}

void launch_clear(const DeviceView* views, uint32_t nviews, uint64_t max_pixels, uint32_t* counters,
                  uint32_t counter_words, uint32_t sm_count, cudaStream_t stream, const float* transforms,
                  uint32_t transform_count, float* tdets, float* mvps) {
    const bool skip = max_pixels == 0;
    uint64_t want = (max_pixels / 2 + 255) / 256;
    uint32_t cap = (sm_count * 16 + nviews - 1) / nviews;
    if (cap < 1) cap = 1;
    uint32_t bx = skip ? 1u : (uint32_t)(want < cap ? (want ? want : 1) : cap);
    dim3 grid(bx, nviews);
    if (!tdets || !mvps) transform_count = 0;
    launch_pdl(k_clear, grid, dim3(256), 0, stream, views, counters, counter_words, skip ? 1u : 0u, transforms,
               transform_count, tdets);
}

void launch_finalize(const DeviceView* views, uint32_t nviews, cudaStream_t stream) {
    launch_pdl(k_finalize, dim3((nviews + 127) / 128), dim3(128), 0, stream, views, nviews);
}

}  // namespace vkgv
