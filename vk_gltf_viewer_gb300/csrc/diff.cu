// Adjoint of the textured resolve (an addition with no reference
// implementation; the shading formula is the commented-out
// visbuffer.frag.glsl:29-34 in linear RGB).
//
// Forward, per covered pixel of the visibility buffer, at the pixel centre
// (nx, ny) in fp32 NDC:
//   lambda = l / sum(l),  l = a x b,  a_k = x_k - nx w_k,  b_k = y_k - ny w_k
//   col = sum lambda_k C_k,  uv = sum lambda_k UV_k
//   uv' = R(rot) uv * scale + offset       (transformUv, mesh_common.h.glsl:129-135)
//   tex = bilinear REPEAT sample of the fp32 RGB texture at uv'
//   rgb = col * albedo * tex
// Backward, with g = dL/drgb = 2 scale (rgb - target): the chain rule through
// the texture's bilinear weights (texel gradients and d tex / d uv'), the
// uv transform, the attribute interpolation (colour gradients), the
// normalisation of lambda, the cross product and the clip transform
// (position gradients).  Gradients are accumulated with fp32 atomics; the
// visibility is the one the raster recomputes in the same call.
#include "kernels.cuh"

namespace vkgv {

namespace {

// Builds the internal raster scene of a differentiable mesh: the vertex
// stream from the fp32 positions, one draw per meshlet, an identity node
// transform, one primitive and one material.
__global__ void k_diff_setup(DiffSetup S) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (uint32_t i = tid; i < S.vertex_count; i += stride) {
        vkgv_vertex v;
        v.position[0] = S.positions[3 * i];
        v.position[1] = S.positions[3 * i + 1];
        v.position[2] = S.positions[3 * i + 2];
        v.color[0] = v.color[1] = v.color[2] = v.color[3] = 255;
        v.normal[0] = v.normal[1] = v.normal[2] = 127;
        v._pad = 0;
        v.uv[0] = v.uv[1] = 0;
        S.vertices[i] = v;
        const float* c = S.colors + 3 * (size_t)i;
        const float* t = S.uvs + 2 * (size_t)i;
        S.vpack[2 * (size_t)i] = make_float4(v.position[0], v.position[1], v.position[2], c[0]);
        S.vpack[2 * (size_t)i + 1] = make_float4(c[1], c[2], t[0], t[1]);
    }
    // the three vertex indices of every visibility id, so that a pixel
    // reaches its vertices in one dependent load
    for (uint32_t j = tid; j < (S.meshlet_count << VKGV_TRIANGLE_BITS); j += stride) {
        const uint32_t m = j >> VKGV_TRIANGLE_BITS, t = j & ((1u << VKGV_TRIANGLE_BITS) - 1u);
        const vkgv_meshlet ml = S.meshlets[m];
        if (t >= ml.triangle_count) continue;
        const uint8_t* tri = S.tri_indices + ml.triangle_offset + 3 * t;
        const uint32_t* vidx = S.vertex_indices + ml.vertex_offset;
        S.tri_verts[j] = make_uint4(vidx[tri[0]], vidx[tri[1]], vidx[tri[2]], 0u);
    }
    for (uint32_t i = tid; i < S.meshlet_count; i += stride) S.draws[i] = vkgv_meshlet_draw{0u, i, 0u};
    if (tid < 16) S.transform[tid] = (tid % 5 == 0) ? 1.0f : 0.0f;
    if (tid == 0) {
        vkgv_primitive pr{};
        pr.vertex_index_buffer = reinterpret_cast<uint64_t>(S.vertex_indices);
        pr.primitive_index_buffer = reinterpret_cast<uint64_t>(S.tri_indices);
        pr.vertex_buffer = reinterpret_cast<uint64_t>(S.vertices);
        pr.meshlet_buffer = reinterpret_cast<uint64_t>(S.meshlets);
        pr.meshlet_count = S.meshlet_count;
        pr.material_index = 0;
        *S.primitive = pr;
        vkgv_material mt{};
        mt.albedo_factor[0] = mt.albedo_factor[1] = mt.albedo_factor[2] = mt.albedo_factor[3] = 1.0f;
        mt.albedo_index = VKGV_INVALID_HANDLE;
        mt.uv_scale[0] = mt.uv_scale[1] = 1.0f;
        mt.double_sided = S.double_sided;
        *S.material = mt;
        *S.cone_table = reinterpret_cast<uint64_t>(S.cones);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Unit normal of triangle t of a meshlet in double; false when degenerate.
__device__ __forceinline__ bool tri_normal(const DiffSetup& S, const uint32_t* vidx, const uint8_t* tri, uint32_t t,
                                           double n[3]) {
    const float* a = S.positions + 3 * (size_t)vidx[tri[3 * t]];
    const float* b = S.positions + 3 * (size_t)vidx[tri[3 * t + 1]];
    const float* c = S.positions + 3 * (size_t)vidx[tri[3 * t + 2]];
    double e1[3], e2[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e1[k] = (double)b[k] - (double)a[k];
        e2[k] = (double)c[k] - (double)a[k];
    }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(len > 1e-30)) return false;
    n[0] /= len, n[1] /= len, n[2] /= len;
    return true;
}

// One warp per meshlet: a normal cone that bounds every triangle normal of
// the meshlet at its current positions (the construction of the scene
// builder: double-precision normals, axis = normalised mean, cutoff = the
// smallest cosine against the rounded float axis less 1e-6, rounded down;
// centre = the AABB centre, radius rounded up), or cutoff -1 (no culling)
// for a degenerate triangle or a spread of normals beyond cos > 0.05.
__global__ void k_diff_cones(DiffSetup S) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < S.meshlet_count; m += warps) {
        const vkgv_meshlet ml = S.meshlets[m];
        const uint32_t vc = min((uint32_t)ml.vertex_count, (uint32_t)VKGV_MAX_VERTICES);
        const uint32_t tc = min((uint32_t)ml.triangle_count, (uint32_t)VKGV_MAX_PRIMITIVES);
        const uint32_t* vidx = S.vertex_indices + ml.vertex_offset;
        const uint8_t* tri = S.tri_indices + ml.triangle_offset;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t k = lane; k < vc; k += 32) {
            const float* p = S.positions + 3 * (size_t)vidx[k];
#pragma unroll
            for (int c = 0; c < 3; ++c) lo[c] = fmin(lo[c], (double)p[c]), hi[c] = fmax(hi[c], (double)p[c]);
        }
        float center[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = warp_min(lo[c]);
            hi[c] = -warp_min(-hi[c]);
            center[c] = (float)(0.5 * (lo[c] + hi[c]));
        }
        double r2 = 0.0;
        for (uint32_t k = lane; k < vc; k += 32) {
            const float* p = S.positions + 3 * (size_t)vidx[k];
            double d2 = 0.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double e = (double)p[c] - (double)center[c];
                d2 += e * e;
            }
            r2 = fmax(r2, d2);
        }
        r2 = -warp_min(-r2);
        vkgv_meshlet_cone cone;
        cone.center[0] = center[0], cone.center[1] = center[1], cone.center[2] = center[2];
        cone.radius = nextafterf((float)(sqrt(r2) * (1.0 + 1e-6) + 1e-7), INFINITY);
        cone.axis[0] = cone.axis[1] = cone.axis[2] = 0.0f;
        cone.cutoff = -1.0f;
        double sum[3] = {0.0, 0.0, 0.0};
        bool degenerate = false;
        for (uint32_t t = lane; t < tc; t += 32) {
            double n[3];
            if (!tri_normal(S, vidx, tri, t, n)) {
                degenerate = true;
            } else {
                sum[0] += n[0], sum[1] += n[1], sum[2] += n[2];
            }
        }
        degenerate = __any_sync(0xffffffffu, degenerate);
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[c] = warp_sum(sum[c]);
        const double sl = sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
        if (!degenerate && sl > 1e-12) {
            const double axis[3] = {sum[0] / sl, sum[1] / sl, sum[2] / sl};
            const float fa[3] = {(float)axis[0], (float)axis[1], (float)axis[2]};
            const double fal = sqrt((double)fa[0] * fa[0] + (double)fa[1] * fa[1] + (double)fa[2] * fa[2]);
            double cmin = 1.0, cmin_f = 1.0;
            for (uint32_t t = lane; t < tc; t += 32) {
                double n[3];
                tri_normal(S, vidx, tri, t, n);
                cmin = fmin(cmin, n[0] * axis[0] + n[1] * axis[1] + n[2] * axis[2]);
                cmin_f = fmin(cmin_f, (n[0] * fa[0] + n[1] * fa[1] + n[2] * fa[2]) / fal);
            }
            cmin = warp_min(cmin);
            cmin_f = warp_min(cmin_f) - 1e-6;
            if (cmin > 0.05 && cmin_f > 0.05) {
                cone.axis[0] = fa[0], cone.axis[1] = fa[1], cone.axis[2] = fa[2];
                cone.cutoff = nextafterf((float)cmin_f, -INFINITY);
            }
        }
        if (lane == 0) S.cones[m] = cone;
    }
}

__device__ __forceinline__ int wrap(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

// Error-free transformations (Dekker / Knuth) for the compensated clip-space
// setup: x * y = p + e exactly, and x + y = s + e exactly.
__device__ __forceinline__ void two_prod(float x, float y, float& p, float& e) {
    p = __fmul_rn(x, y);
    e = __fmaf_rn(x, y, -p);
}

__device__ __forceinline__ void two_sum(float x, float y, float& s, float& e) {
    s = __fadd_rn(x, y);
    const float bb = __fsub_rn(s, x);
    e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(y, bb));
}

// Row j of the column-major M applied to (x, y, z, 1) as an unevaluated sum
// hi + lo accurate to about twice fp32 precision (the compensated dot
// product of Ogita, Rump and Oishi, "Accurate sum and dot product", 2005).
__device__ __forceinline__ void dot_df(const float* M, int j, float x, float y, float z, float& hi, float& lo) {
    float s = M[12 + j], err = 0.0f, p, e, q;
    two_prod(M[j], x, p, e);
    two_sum(s, p, s, q);
    err = __fadd_rn(err, __fadd_rn(q, e));
    two_prod(M[4 + j], y, p, e);
    two_sum(s, p, s, q);
    err = __fadd_rn(err, __fadd_rn(q, e));
    two_prod(M[8 + j], z, p, e);
    two_sum(s, p, s, q);
    err = __fadd_rn(err, __fadd_rn(q, e));
    two_sum(s, err, hi, lo);
}

// a = x - nx w and b = y - ny w of one vertex, each rounded once from an
// almost exact value.  a and b vanish where the pixel ray passes near the
// vertex; there the plain fp32 form loses most of its digits to
// cancellation, and the position gradient (through l = a x b) inherits
// the loss.
__device__ __forceinline__ void clip_ab(const float* VP, const float* q, float nx, float ny, float& a, float& b) {
    float xh, xl, yh, yl, wh, wl;
    dot_df(VP, 0, q[0], q[1], q[2], xh, xl);
    dot_df(VP, 1, q[0], q[1], q[2], yh, yl);
    dot_df(VP, 3, q[0], q[1], q[2], wh, wl);
    a = __fadd_rn(__fmaf_rn(-nx, wh, xh), __fmaf_rn(-nx, wl, xl));
    b = __fadd_rn(__fmaf_rn(-ny, wh, yh), __fmaf_rn(-ny, wl, yl));
}

// One pixel of the forward image (BACKWARD = false) or of the gradient pass.
template <bool BACKWARD>
__device__ __forceinline__ void shade_pixel(const DiffArgs& A, const DeviceView& V, const float* VP, float sn, float cs,
                                            uint32_t p, float& loss_acc) {
    const uint32_t w = V.w;
    const uint32_t lo = (uint32_t)V.depth_id[p];
    float tgt[3] = {0.0f, 0.0f, 0.0f};
    const bool mse = V.diff_target != nullptr;
    if (BACKWARD && mse) {
        tgt[0] = V.diff_target[3 * p];
        tgt[1] = V.diff_target[3 * p + 1];
        tgt[2] = V.diff_target[3 * p + 2];
    }
    if (lo == 0) {
        if (BACKWARD) loss_acc += A.scale * (tgt[0] * tgt[0] + tgt[1] * tgt[1] + tgt[2] * tgt[2]);
        else if (V.diff_rgb) V.diff_rgb[3 * p] = V.diff_rgb[3 * p + 1] = V.diff_rgb[3 * p + 2] = 0.0f;
        return;
    }
    const uint4 tvi = A.tri_verts[lo - 1u];
    // The sample point is the fp32 NDC of the pixel centre.
    const float nx = fsub(fmul(fdiv(fadd((float)(p % w), 0.5f), (float)V.w), 2.0f), 1.0f);
    const float ny = fsub(fmul(fdiv(fadd((float)(p / w), 0.5f), (float)V.h), 2.0f), 1.0f);
    const uint32_t vi[3] = {tvi.x, tvi.y, tvi.z};
    float4 P0[3], P1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        P0[k] = A.vpack[2 * (size_t)vi[k]];
        P1[k] = A.vpack[2 * (size_t)vi[k] + 1];
    }
    // a and b from the compensated clip transform in both passes: on a
    // sub-pixel triangle whose UVs span a large part of the texture (around
    // the poles and the u seam of an equirectangular map) the plain fp32
    // form's barycentric error becomes a texel-sized UV error in the
    // forward image too.
    float a[3], b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float q[3] = {P0[k].x, P0[k].y, P0[k].z};
        clip_ab(VP, q, nx, ny, a[k], b[k]);
    }
    float l[3] = {fsub(fmul(a[1], b[2]), fmul(a[2], b[1])), fsub(fmul(a[2], b[0]), fmul(a[0], b[2])),
                  fsub(fmul(a[0], b[1]), fmul(a[1], b[0]))};
    const float sum = fadd(fadd(l[0], l[1]), l[2]);
    if (!(sum != 0.0f)) {  // degenerate: shaded as empty, no gradient
        if (BACKWARD) loss_acc += A.scale * (tgt[0] * tgt[0] + tgt[1] * tgt[1] + tgt[2] * tgt[2]);
        else if (V.diff_rgb) V.diff_rgb[3 * p] = V.diff_rgb[3 * p + 1] = V.diff_rgb[3 * p + 2] = 0.0f;
        return;
    }
    float lam[3] = {fdiv(l[0], sum), fdiv(l[1], sum), fdiv(l[2], sum)};
    float C[3][3], UV[3][2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        C[k][0] = P0[k].w, C[k][1] = P1[k].x, C[k][2] = P1[k].y;
        UV[k][0] = P1[k].z, UV[k][1] = P1[k].w;
    }
    float col[3], uv[2];
#pragma unroll
    for (int j = 0; j < 3; ++j)
        col[j] = fadd(fadd(fmul(lam[0], C[0][j]), fmul(lam[1], C[1][j])), fmul(lam[2], C[2][j]));
#pragma unroll
    for (int j = 0; j < 2; ++j)
        uv[j] = fadd(fadd(fmul(lam[0], UV[0][j]), fmul(lam[1], UV[1][j])), fmul(lam[2], UV[2][j]));
    const float ru = fadd(fmul(cs, uv[0]), fmul(sn, uv[1]));
    const float rv = fadd(fmul(-sn, uv[0]), fmul(cs, uv[1]));
    const float tu = fadd(fmul(ru, A.uv_scale[0]), A.uv_offset[0]);
    const float tv = fadd(fmul(rv, A.uv_scale[1]), A.uv_offset[1]);
    const float tx = fsub(fmul(tu, (float)A.tex_w), 0.5f), ty = fsub(fmul(tv, (float)A.tex_h), 0.5f);
    const float fx = floorf(tx), fy = floorf(ty);
    const float ax = fsub(tx, fx), ay = fsub(ty, fy);
    const int x0 = wrap((int)fx, (int)A.tex_w), x1 = wrap((int)fx + 1, (int)A.tex_w);
    const int y0 = wrap((int)fy, (int)A.tex_h), y1 = wrap((int)fy + 1, (int)A.tex_h);
    const size_t i00 = 3 * ((size_t)y0 * A.tex_w + x0), i01 = 3 * ((size_t)y0 * A.tex_w + x1);
    const size_t i10 = 3 * ((size_t)y1 * A.tex_w + x0), i11 = 3 * ((size_t)y1 * A.tex_w + x1);
    float T00[3], T01[3], T10[3], T11[3], tex[3], rgb[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        T00[j] = A.texture[i00 + j];
        T01[j] = A.texture[i01 + j];
        T10[j] = A.texture[i10 + j];
        T11[j] = A.texture[i11 + j];
        const float top = fadd(T00[j], fmul(ax, fsub(T01[j], T00[j])));
        const float bot = fadd(T10[j], fmul(ax, fsub(T11[j], T10[j])));
        tex[j] = fadd(top, fmul(ay, fsub(bot, top)));
        rgb[j] = fmul(fmul(col[j], A.albedo[j]), tex[j]);
    }
    if (!BACKWARD) {
        if (V.diff_rgb) {
            V.diff_rgb[3 * p] = rgb[0];
            V.diff_rgb[3 * p + 1] = rgb[1];
            V.diff_rgb[3 * p + 2] = rgb[2];
        }
        return;
    }
    // ---- backward
    float g[3], dcol[3], dtex[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (mse) {
            const float r = rgb[j] - tgt[j];
            loss_acc += A.scale * r * r;
            g[j] = 2.0f * A.scale * r;
        } else {
            g[j] = V.diff_grad[3 * p + j];
        }
        dcol[j] = g[j] * A.albedo[j] * tex[j];
        dtex[j] = g[j] * col[j] * A.albedo[j];
    }
    if (A.acc_tex) {
        const float w00 = (1.0f - ax) * (1.0f - ay), w01 = ax * (1.0f - ay);
        const float w10 = (1.0f - ax) * ay, w11 = ax * ay;
        atomicAdd(A.acc_tex + i00 / 3, make_float4(dtex[0] * w00, dtex[1] * w00, dtex[2] * w00, 0.0f));
        atomicAdd(A.acc_tex + i01 / 3, make_float4(dtex[0] * w01, dtex[1] * w01, dtex[2] * w01, 0.0f));
        atomicAdd(A.acc_tex + i10 / 3, make_float4(dtex[0] * w10, dtex[1] * w10, dtex[2] * w10, 0.0f));
        atomicAdd(A.acc_tex + i11 / 3, make_float4(dtex[0] * w11, dtex[1] * w11, dtex[2] * w11, 0.0f));
    }
    // d tex / d uv' through the bilinear weights
    float dtu = 0.0f, dtv = 0.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        dtu += dtex[j] * ((1.0f - ay) * (T01[j] - T00[j]) + ay * (T11[j] - T10[j]));
        dtv += dtex[j] * ((1.0f - ax) * (T10[j] - T00[j]) + ax * (T11[j] - T01[j]));
    }
    dtu *= (float)A.tex_w;
    dtv *= (float)A.tex_h;
    const float dru = dtu * A.uv_scale[0], drv = dtv * A.uv_scale[1];
    const float du = cs * dru - sn * drv, dv = sn * dru + cs * drv;
    float dlam[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        dlam[k] = dcol[0] * C[k][0] + dcol[1] * C[k][1] + dcol[2] * C[k][2] + du * UV[k][0] + dv * UV[k][1];
        if (A.acc_col)
            atomicAdd(A.acc_col + vi[k], make_float4(dcol[0] * lam[k], dcol[1] * lam[k], dcol[2] * lam[k], 0.0f));
    }
    if (!A.acc_pos) return;
    const float dot = lam[0] * dlam[0] + lam[1] * dlam[1] + lam[2] * dlam[2];
    const float dl[3] = {(dlam[0] - dot) / sum, (dlam[1] - dot) / sum, (dlam[2] - dot) / sum};
    // l = a x b: dL/da = b x dl, dL/db = dl x a
    const float da[3] = {b[1] * dl[2] - b[2] * dl[1], b[2] * dl[0] - b[0] * dl[2], b[0] * dl[1] - b[1] * dl[0]};
    const float db[3] = {dl[1] * a[2] - dl[2] * a[1], dl[2] * a[0] - dl[0] * a[2], dl[0] * a[1] - dl[1] * a[0]};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float dx = da[k], dy = db[k], dw = -nx * da[k] - ny * db[k];
        atomicAdd(A.acc_pos + vi[k], make_float4(VP[0] * dx + VP[1] * dy + VP[3] * dw,
                                                 VP[4] * dx + VP[5] * dy + VP[7] * dw,
                                                 VP[8] * dx + VP[9] * dy + VP[11] * dw, 0.0f));
    }
}

// One thread per pixel over a (max pixels / 256, views) grid: for views past
// kShadeMaxViews.
template <bool BACKWARD>
__global__ void __launch_bounds__(256) k_diff_shade(DiffArgs A, const DeviceView* __restrict__ views) {
    const DeviceView& V = views[blockIdx.y];
    const uint32_t n = V.w * V.h;
    float VP[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) VP[k] = V.cam->view_projection[k];
    float sn, cs;
    sincosf(A.uv_rotation, &sn, &cs);
    float loss_acc = 0.0f;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        shade_pixel<BACKWARD>(A, V, VP, sn, cs, p, loss_acc);
    if (BACKWARD && A.loss) {
        // warp-reduce the loss, one atomic per warp
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(A.loss, loss_acc);
    }
}

// Persistent form: one wave of resident CTAs whose warps take chunks of
// kShadeChunk pixels (all views' chunks numbered in view order) from a
// global counter, so warps of background pixels neither retire early (which
// left the SMs below their register-limited residency) nor wait at a CTA
// barrier for warps of covered pixels, and views smaller than the largest
// cost no empty CTAs.  The last CTA to finish returns the counters to zero.
constexpr uint32_t kShadeChunk = 512;
constexpr uint32_t kShadeMaxViews = 4096;

template <bool BACKWARD>
__global__ void __launch_bounds__(256, 3) k_diff_shade_chunks(DiffArgs A, const DeviceView* __restrict__ views,
                                                           uint32_t nviews, uint32_t* work) {
    __shared__ uint32_t s_pre[kShadeMaxViews + 1];
    for (uint32_t v = threadIdx.x; v < nviews; v += blockDim.x)
        s_pre[v + 1] = (views[v].w * views[v].h + kShadeChunk - 1) / kShadeChunk;
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
    float sn, cs;
    sincosf(A.uv_rotation, &sn, &cs);
    float VP[16];
    uint32_t cur = 0xffffffffu;
    float loss_acc = 0.0f;
    for (;;) {
        // each warp takes its own chunks: no CTA barrier holds a warp of
        // background pixels behind one of covered pixels
        uint32_t item = 0;
        if ((threadIdx.x & 31u) == 0) item = atomicAdd(work, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        // the view holding the chunk: the last v with s_pre[v] <= item
        uint32_t v = 0, hi = nviews;
        while (v + 1 < hi) {
            const uint32_t mid = (v + hi) >> 1;
            if (s_pre[mid] <= item) v = mid;
            else hi = mid;
        }
        const DeviceView& V = views[v];
        if (v != cur) {
            cur = v;
#pragma unroll
            for (int k = 0; k < 16; ++k) VP[k] = V.cam->view_projection[k];
        }
        const uint32_t n = V.w * V.h, base = (item - s_pre[v]) * kShadeChunk;
        // two pixels per step: the compiler interleaves their load chains
        // (id -> vertex triple -> vertex records -> texels), and the kernel
        // then fits 80 registers, three CTAs per SM (C5 step -1.2%)
#pragma unroll 2
        for (uint32_t j = threadIdx.x & 31u; j < kShadeChunk; j += 32) {
            const uint32_t p = base + j;
            if (p < n) shade_pixel<BACKWARD>(A, V, VP, sn, cs, p, loss_acc);
        }
    }
    if (BACKWARD && A.loss) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(A.loss, loss_acc);
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

// grad[3 i + j] += acc[i].{x, y, z}
__global__ void k_diff_scatter(const float4* __restrict__ acc, float* __restrict__ grad, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        grad[3 * (size_t)i] += a.x;
        grad[3 * (size_t)i + 1] += a.y;
        grad[3 * (size_t)i + 2] += a.z;
    }
}

void scatter(const float4* acc, float* grad, uint32_t n, cudaStream_t stream) {
    if (!acc || !grad || n == 0) return;
    uint32_t blocks = (n + 255) / 256;
    blocks = blocks < 8192 ? blocks : 8192;
    k_diff_scatter<<<blocks, 256, 0, stream>>>(acc, grad, n);
}

}  // namespace

void launch_diff_setup(const DiffSetup& S, cudaStream_t stream) {
    const uint32_t n = S.vertex_count > S.meshlet_count ? S.vertex_count : S.meshlet_count;
    uint32_t blocks = (n + 255) / 256;
    blocks = blocks ? (blocks < 4096 ? blocks : 4096) : 1;
    k_diff_setup<<<blocks, 256, 0, stream>>>(S);
}

void launch_diff_cones(const DiffSetup& S, cudaStream_t stream) {
    uint32_t blocks = (S.meshlet_count * 32 + 255) / 256;
    blocks = blocks ? (blocks < 8192 ? blocks : 8192) : 1;
    k_diff_cones<<<blocks, 256, 0, stream>>>(S);
}

void launch_diff_scatter(const DiffArgs& A, cudaStream_t stream) {
    scatter(A.acc_pos, A.grad_positions, A.vertex_count, stream);
    scatter(A.acc_col, A.grad_colors, A.vertex_count, stream);
    scatter(A.acc_tex, A.grad_texture, A.tex_w * A.tex_h, stream);
}

void launch_diff_shade(const DiffArgs& A, const DeviceView* views, uint32_t nviews, uint64_t max_px, bool backward,
                       uint32_t* work, uint32_t sm_count, cudaStream_t stream) {
    if (nviews <= kShadeMaxViews && work) {
        int per_sm = 0;
        const cudaError_t e = backward
            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diff_shade_chunks<true>, 256, 0)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diff_shade_chunks<false>, 256, 0);
        if (e == cudaSuccess && per_sm > 0) {
            const uint32_t blocks = sm_count * (uint32_t)per_sm;
            if (backward)
                k_diff_shade_chunks<true><<<blocks, 256, 0, stream>>>(A, views, nviews, work);
            else
                k_diff_shade_chunks<false><<<blocks, 256, 0, stream>>>(A, views, nviews, work);
            return;
        }
        cudaGetLastError();
    }
    uint32_t bx = (uint32_t)((max_px + 255) / 256);
    if (bx > 65535u) bx = 65535u;
    if (bx == 0) bx = 1;
    dim3 grid(bx, nviews);
    if (backward)
        k_diff_shade<true><<<grid, 256, 0, stream>>>(A, views);
    else
        k_diff_shade<false><<<grid, 256, 0, stream>>>(A, views);
}

}  // namespace vkgv
