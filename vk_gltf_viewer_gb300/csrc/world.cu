// The node tree on the device: animation sampling, world transforms and the
// MeshletDraw list (src/vk_gltf_viewer/world.cpp:187-345,
// include/vk_gltf_viewer/assets.hpp:51-113).
//
// The reference walks the tree on the host every frame (World::iterateNode),
// sampling every channel of every animation for every node, composing
// parent * T * R * S, and copies the transforms (and, on a scene change, the
// draw list) into mapped buffers.  Here the host walks the tree once
// (plan_world) and each frame is two kernels:
//   k_world_local  one thread per node: rest TRS, the node's channels in
//                  application order, local matrix T * R * S;
//   k_world_chain  one thread per transform slot: the product of the local
//                  matrices from the root down its path, in the reference's
//                  association order ((I * L_root) * ...) * L_node.
// The draw list is k_world_draws: one block per tile of 1024 draws whose
// first segment the plan holds, the tile's records staged in shared memory
// and stored as 16-byte words.
//
// Arithmetic the reference leaves to fastgltf (absent from the reference
// tree; no pinned version) is restated from the glTF 2.0 specification's
// animation appendix and pinned here and in the oracle:
//   lerp   (1 - t) * a + t * b
//   slerp  a * sin((1 - t) θ) / sin θ + b' * sin(t θ) / sin θ in float,
//          b' = b or -b for the shorter arc, θ from the half-angle identities
//          |a - b'| = 2 sin(θ/2), |a + b'| = 2 cos(θ/2) and a power series
//          for asin at θ/4; sin by its Taylor series (both below, accurate
//          to about one ulp; float64 would run on GB300's narrow FP64 pipe);
//          (1 - t) a + t b' when θ < 1e-6
//   cubic  the Hermite form of assets.hpp:93-108 with t² = t * t and
//          t³ = t² * t; rotations normalised by v / sqrt(dot(v, v))
//   TRS    the rotation matrix of a unit quaternion (glTF's
//          node transform), columns scaled by S, translation in column 3.
#include <algorithm>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace vkgv {

namespace {

// Taylor coefficients (-1)^k / (2k+1)!, k = 0..7, rounded to float:
// sin(x) = x * P(x^2) within 1.6e-7 relative on [0, pi/2].
__constant__ float kSinCoef[8] = {0x1.000000p+0f,  -0x1.555556p-3f, 0x1.111112p-7f,  -0x1.a01a02p-13f,
                                  0x1.71de3ap-19f, -0x1.ae6456p-26f, 0x1.612462p-33f, -0x1.ae7f3ep-41f};

// asin(z) = z * sum_n c_n z^(2n), c_n = C(2n, n) / (4^n (2n + 1)), n = 0..9,
// rounded to float; within 1.2e-7 relative for z <= sin(pi/8).
__constant__ float kAsinCoef[10] = {0x1.000000p+0f, 0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f,
                                    0x1.f1c71cp-6f, 0x1.6e8ba2p-6f, 0x1.1c4ec4p-6f, 0x1.c9999ap-7f,
                                    0x1.7a8788p-7f, 0x1.3fde50p-7f};

__device__ float sin_series(float x) {
    const float u = fmul(x, x);
    float p = kSinCoef[7];
#pragma unroll
    for (int k = 6; k >= 0; --k) p = fadd(fmul(p, u), kSinCoef[k]);
    return fmul(x, p);
}

__device__ float asin_series(float z) {
    const float u = fmul(z, z);
    float p = kAsinCoef[9];
#pragma unroll
    for (int k = 8; k >= 0; --k) p = fadd(fmul(p, u), kAsinCoef[k]);
    return fmul(z, p);
}

__device__ void slerp(const float* a, const float* b, float t, float out[4]) {
    float A[4], B[4];
    for (int k = 0; k < 4; ++k) A[k] = a[k], B[k] = b[k];
    const float d = fadd(fadd(fadd(fmul(A[0], B[0]), fmul(A[1], B[1])), fmul(A[2], B[2])), fmul(A[3], B[3]));
    if (d < 0.0f)
        for (int k = 0; k < 4; ++k) B[k] = -B[k];
    float sd = 0.0f, sp = 0.0f;
    for (int k = 0; k < 4; ++k) {
        const float m = fsub(A[k], B[k]), p = fadd(A[k], B[k]);
        sd = fadd(sd, fmul(m, m));
        sp = fadd(sp, fmul(p, p));
    }
    const float s = fmul(0.5f, __fsqrt_rn(sd));  // sin(theta / 2)
    const float c = fmul(0.5f, __fsqrt_rn(sp));  // cos(theta / 2)
    const float z = fdiv(s, __fsqrt_rn(fmul(2.0f, fadd(1.0f, c))));  // sin(theta / 4)
    const float theta = fmul(4.0f, asin_series(z));
    float w0 = fsub(1.0f, t), w1 = t;
    if (theta >= 1e-6f) {
        const float sn = sin_series(theta);
        if (sn != 0.0f) {
            w0 = fdiv(sin_series(fmul(fsub(1.0f, t), theta)), sn);
            w1 = fdiv(sin_series(fmul(t, theta)), sn);
        }
    }
    for (int k = 0; k < 4; ++k) out[k] = fadd(fmul(w0, A[k]), fmul(w1, B[k]));
}

// AnimationSampler::sample (assets.hpp:56-113) at `time`; writes `components`
// floats.
__device__ void sample(const WorldSampler& S, const float* __restrict__ keys, float time, uint32_t path,
                       float out[4]) {
    const float* in = keys + S.input;
    const float* val = keys + S.output;
    const uint32_t n = S.input_count, cc = S.components;
    const bool cubic = S.interpolation == VKGV_INTERP_CUBICSPLINE;
    const float tt = fmodf(time, in[n - 1]);  // loops the animation (assets.hpp:61)
    uint32_t lo = 0, hi = n;                  // std::lower_bound
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (in[mid] < tt)
            lo = mid + 1;
        else
            hi = mid;
    }
    const float* src;
    if (lo == 0) {
        src = val + (cubic ? 1u : 0u) * cc;
    } else if (lo == n) {
        src = val + (cubic ? S.output_count - 2u : S.output_count - 1u) * cc;
    } else {
        const uint32_t i = lo;
        const float t = fdiv(fsub(tt, in[i - 1]), fsub(in[i], in[i - 1]));
        if (S.interpolation == VKGV_INTERP_STEP) {
            src = val + (i - 1) * cc;
        } else if (S.interpolation == VKGV_INTERP_LINEAR) {
            const float* a = val + (i - 1) * cc;
            const float* b = val + i * cc;
            if (path == VKGV_PATH_ROTATION) {
                slerp(a, b, t, out);
            } else {
                const float u = fsub(1.0f, t);
                for (uint32_t k = 0; k < cc; ++k) out[k] = fadd(fmul(u, a[k]), fmul(t, b[k]));
            }
            return;
        } else {
            const float t2 = fmul(t, t), t3 = fmul(t2, t);
            const float dt = fsub(in[i], in[i - 1]);
            const float h00 = fadd(fsub(fmul(2.0f, t3), fmul(3.0f, t2)), 1.0f);
            const float h10 = fadd(fsub(t3, fmul(2.0f, t2)), t);
            const float h01 = fadd(fmul(-2.0f, t3), fmul(3.0f, t2));
            const float h11 = fsub(t3, t2);
            const float* p0 = val + (3 * (i - 1) + 1) * cc;
            const float* m0 = val + (3 * (i - 1) + 2) * cc;
            const float* p1 = val + (3 * i + 1) * cc;
            const float* m1 = val + (3 * i + 0) * cc;
            for (uint32_t k = 0; k < cc; ++k)
                out[k] = fadd(fadd(fadd(fmul(p0[k], h00), fmul(fmul(m0[k], h10), dt)), fmul(p1[k], h01)),
                              fmul(fmul(m1[k], h11), dt));
            if (path == VKGV_PATH_ROTATION) {
                const float len = __fsqrt_rn(
                    fadd(fadd(fadd(fmul(out[0], out[0]), fmul(out[1], out[1])), fmul(out[2], out[2])),
                         fmul(out[3], out[3])));
                for (int k = 0; k < 4; ++k) out[k] = fdiv(out[k], len);
            }
            return;
        }
    }
    for (uint32_t k = 0; k < cc; ++k) out[k] = src[k];
}

// T * R * S of a glTF node, column-major.
__device__ void trs_matrix(const float t[3], const float q[4], const float s[3], float m[16]) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    const float xx = fmul(x, x), yy = fmul(y, y), zz = fmul(z, z);
    const float xy = fmul(x, y), xz = fmul(x, z), yz = fmul(y, z);
    const float wx = fmul(w, x), wy = fmul(w, y), wz = fmul(w, z);
    const float r[9] = {fsub(1.0f, fmul(2.0f, fadd(yy, zz))), fmul(2.0f, fadd(xy, wz)), fmul(2.0f, fsub(xz, wy)),
                        fmul(2.0f, fsub(xy, wz)), fsub(1.0f, fmul(2.0f, fadd(xx, zz))), fmul(2.0f, fadd(yz, wx)),
                        fmul(2.0f, fadd(xz, wy)), fmul(2.0f, fsub(yz, wx)), fsub(1.0f, fmul(2.0f, fadd(xx, yy)))};
    for (int c = 0; c < 3; ++c) {
        for (int j = 0; j < 3; ++j) m[4 * c + j] = fmul(r[3 * c + j], s[c]);
        m[4 * c + 3] = 0.0f;
    }
    m[12] = t[0], m[13] = t[1], m[14] = t[2], m[15] = 1.0f;
}

__global__ void __launch_bounds__(128) k_world_local(WorldArgs W, float time) {
    pdl_begin();
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= W.node_count) return;
    const float* r = W.rest + 10 * (size_t)n;
    float t[3] = {r[0], r[1], r[2]}, q[4] = {r[3], r[4], r[5], r[6]}, s[3] = {r[7], r[8], r[9]};
    // World::iterateNode (world.cpp:187-215): every channel that targets the
    // node, in application order, overrides its path.
    for (uint32_t e = W.chan_offsets[n]; e < W.chan_offsets[n + 1]; ++e) {
        const uint2 ch = W.chans[e];
        float v[4];
        sample(W.samplers[ch.x], W.keys, time, ch.y, v);
        if (ch.y == VKGV_PATH_TRANSLATION)
            t[0] = v[0], t[1] = v[1], t[2] = v[2];
        else if (ch.y == VKGV_PATH_ROTATION)
            q[0] = v[0], q[1] = v[1], q[2] = v[2], q[3] = v[3];
        else
            s[0] = v[0], s[1] = v[1], s[2] = v[2];
    }
    float m[16];
    trs_matrix(t, q, s, m);
    float4* out = reinterpret_cast<float4*>(W.local + 16 * (size_t)n);
    for (int k = 0; k < 4; ++k) out[k] = make_float4(m[4 * k], m[4 * k + 1], m[4 * k + 2], m[4 * k + 3]);
}

__global__ void __launch_bounds__(128) k_world_chain(WorldArgs W, float* __restrict__ transforms) {
    pdl_begin();
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= W.slot_count) return;
    float M[16] = {1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    for (uint32_t k = W.chain_offsets[slot]; k < W.chain_offsets[slot + 1]; ++k) {
        const float4* L4 = reinterpret_cast<const float4*>(W.local + 16 * (size_t)W.chain_nodes[k]);
        float L[16], R[16];
        for (int c = 0; c < 4; ++c) {
            const float4 v = L4[c];
            L[4 * c] = v.x, L[4 * c + 1] = v.y, L[4 * c + 2] = v.z, L[4 * c + 3] = v.w;
        }
        m4m(M, L, R);
        for (int i = 0; i < 16; ++i) M[i] = R[i];
    }
    float4* out = reinterpret_cast<float4*>(transforms + 16 * (size_t)slot);
    for (int k = 0; k < 4; ++k) out[k] = make_float4(M[4 * k], M[4 * k + 1], M[4 * k + 2], M[4 * k + 3]);
}

// Largest s in [lo, hi) with first[s] <= d (first[lo] <= d holds).
__device__ __forceinline__ uint32_t segment_of(const uint32_t* __restrict__ first, uint32_t lo, uint32_t hi,
                                               uint32_t d) {
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(first + mid) <= d)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// One block per tile of kWorldTile draws (kWorldTile / kWorldThreads per
// thread): each thread finds its draws' segments between the tile's first
// and last segment (from the plan), the block stages the tile's
// 3 * kWorldTile words in shared memory and stores them as 16-byte words.
// 1024-draw tiles put the C2 list (824 tiles) in one wave.
__global__ void __launch_bounds__(kWorldThreads) k_world_draws(WorldArgs W, uint32_t* __restrict__ words) {
    pdl_begin();
    __shared__ __align__(16) uint32_t s_words[3 * kWorldTile];
    const uint32_t tile = blockIdx.x, t = threadIdx.x;
    const uint32_t first = tile * kWorldTile;
    const uint32_t count = min(kWorldTile, W.draw_count - first);
    const uint32_t lo = __ldg(W.tile_seg + tile);
    const uint32_t hi = tile + 1 < W.tile_count ? __ldg(W.tile_seg + tile + 1) + 1 : W.seg_count;
#pragma unroll
    for (uint32_t k = 0; k < kWorldTile / kWorldThreads; ++k) {
        const uint32_t i = t + k * kWorldThreads;
        if (i < count) {
            const uint32_t d = first + i;
            const uint32_t seg = segment_of(W.seg_first, lo, hi, d);
            const uint2 info = __ldg(W.seg_info + seg);
            s_words[3 * i] = info.x;
            s_words[3 * i + 1] = d - __ldg(W.seg_first + seg);
            s_words[3 * i + 2] = info.y;
        }
    }
    __syncthreads();
    const uint32_t n = 3 * count;
    uint4* out4 = reinterpret_cast<uint4*>(words + 3ull * first);  // 12 KiB per tile: 16-byte aligned
    for (uint32_t i = t; i < n / 4; i += kWorldThreads) __stcs(out4 + i, reinterpret_cast<const uint4*>(s_words)[i]);
    const uint32_t tail = n & ~3u;
    if (t < n - tail) __stcs(words + 3ull * first + tail + t, s_words[tail + t]);
}

}  // namespace

void launch_world_transforms(const WorldArgs& W, float time, float* transforms, cudaStream_t stream) {
    if (W.node_count) launch_pdl(k_world_local, dim3((W.node_count + 127) / 128), dim3(128), 0, stream, W, time);
    if (W.slot_count)
        launch_pdl(k_world_chain, dim3((W.slot_count + 127) / 128), dim3(128), 0, stream, W, transforms);
}

void launch_world_draws(const WorldArgs& W, uint32_t* draws, uint32_t sm_count, cudaStream_t stream) {
    (void)sm_count;
    if (!W.draw_count) return;
    launch_pdl(k_world_draws, dim3(W.tile_count), dim3(kWorldThreads), 0, stream, W, draws);
}

// ------------------------------------------------------------- host plan

int plan_world(const vkgv_world_desc& D, WorldPlan& P, std::string& err) {
    auto bad = [&](const std::string& m) {
        err = m;
        return (int)VKGV_INVALID_ARG;
    };
    if (D.node_count && !D.nodes) return bad("nodes is NULL");
    if (D.child_count && !D.children) return bad("children is NULL");
    if (D.root_count && !D.roots) return bad("roots is NULL");
    if (D.mesh_count && (!D.mesh_offsets || !D.mesh_primitives)) return bad("mesh tables are NULL");
    if (D.primitive_count && !D.primitive_meshlet_counts) return bad("primitive_meshlet_counts is NULL");
    if (D.sampler_count && !D.samplers) return bad("samplers is NULL");
    if (D.channel_count && !D.channels) return bad("channels is NULL");
    const uint32_t N = D.node_count;
    for (uint32_t n = 0; n < N; ++n) {
        const vkgv_node& nd = D.nodes[n];
        if ((uint64_t)nd.first_child + nd.child_count > D.child_count) return bad("node children out of range");
        if (nd.mesh_index != VKGV_INVALID_HANDLE && nd.mesh_index >= D.mesh_count) return bad("mesh_index out of range");
    }
    for (uint32_t c = 0; c < D.child_count; ++c)
        if (D.children[c] >= N) return bad("child index out of range");
    for (uint32_t r = 0; r < D.root_count; ++r)
        if (D.roots[r] >= N) return bad("root index out of range");
    for (uint32_t m = 0; m < D.mesh_count; ++m)
        if (D.mesh_offsets[m] > D.mesh_offsets[m + 1]) return bad("mesh_offsets must not decrease");
    const uint32_t mp_count = D.mesh_count ? D.mesh_offsets[D.mesh_count] : 0;
    for (uint32_t i = 0; i < mp_count; ++i)
        if (D.mesh_primitives[i] >= D.primitive_count) return bad("mesh primitive index out of range");

    // samplers: validate and pool the keyframes
    P.samplers.assign(D.sampler_count, WorldSampler{});
    P.keys.clear();
    for (uint32_t i = 0; i < D.sampler_count; ++i) {
        const vkgv_anim_sampler& s = D.samplers[i];
        if (s.input_count == 0 || !s.input || !s.output) return bad("sampler without keyframes");
        if (s.interpolation > VKGV_INTERP_CUBICSPLINE) return bad("unknown interpolation");
        if (s.components < 1 || s.components > 4) return bad("sampler components must be 1 to 4");
        const uint64_t want = (uint64_t)s.input_count * (s.interpolation == VKGV_INTERP_CUBICSPLINE ? 3u : 1u);
        if (s.output_count != want) return bad("sampler output_count does not match its keyframes");
        const uint64_t total = P.keys.size() + s.input_count + (uint64_t)s.output_count * s.components;
        if (total >= (1ull << 32)) {
            err = "keyframe data exceeds 2^32 floats";
            return VKGV_LIMIT_EXCEEDED;
        }
        WorldSampler& w = P.samplers[i];
        w.input = (uint32_t)P.keys.size();
        P.keys.insert(P.keys.end(), s.input, s.input + s.input_count);
        w.output = (uint32_t)P.keys.size();
        P.keys.insert(P.keys.end(), s.output, s.output + (size_t)s.output_count * s.components);
        w.input_count = s.input_count;
        w.output_count = s.output_count;
        w.interpolation = s.interpolation;
        w.components = s.components;
    }
    // channels per node, in application order; weights and untargeted
    // channels do nothing (world.cpp:190-213)
    P.chan_offsets.assign(N + 1, 0);
    for (uint32_t c = 0; c < D.channel_count; ++c) {
        const vkgv_anim_channel& ch = D.channels[c];
        if (ch.path < VKGV_PATH_TRANSLATION || ch.path > VKGV_PATH_WEIGHTS) return bad("unknown channel path");
        if (ch.node == VKGV_INVALID_HANDLE || ch.path == VKGV_PATH_WEIGHTS) continue;
        if (ch.node >= N) return bad("channel node out of range");
        if (ch.sampler >= D.sampler_count) return bad("channel sampler out of range");
        const uint32_t want = ch.path == VKGV_PATH_ROTATION ? 4u : 3u;
        if (D.samplers[ch.sampler].components != want) return bad("sampler components do not match the path");
        ++P.chan_offsets[ch.node + 1];
    }
    for (uint32_t n = 0; n < N; ++n) P.chan_offsets[n + 1] += P.chan_offsets[n];
    P.chans.assign(P.chan_offsets[N], make_uint2(0, 0));
    {
        std::vector<uint32_t> fill(P.chan_offsets.begin(), P.chan_offsets.end() - 1);
        for (uint32_t c = 0; c < D.channel_count; ++c) {
            const vkgv_anim_channel& ch = D.channels[c];
            if (ch.node == VKGV_INVALID_HANDLE || ch.path == VKGV_PATH_WEIGHTS) continue;
            P.chans[fill[ch.node]++] = make_uint2(ch.sampler, ch.path);
        }
    }
    P.rest.resize((size_t)N * 10);
    for (uint32_t n = 0; n < N; ++n) {
        const vkgv_node& nd = D.nodes[n];
        float* r = &P.rest[(size_t)n * 10];
        for (int k = 0; k < 3; ++k) r[k] = nd.translation[k];
        for (int k = 0; k < 4; ++k) r[3 + k] = nd.rotation[k];
        for (int k = 0; k < 3; ++k) r[7 + k] = nd.scale[k];
    }

    // depth-first walk from the roots (World::iterateNode): a node with a
    // mesh takes the next transform slot; its path is the slot's chain
    P.chain_offsets.assign(1, 0);
    P.chain_nodes.clear();
    P.seg_first.assign(1, 0);
    P.seg_info.clear();
    uint64_t draws = 0, visits = 0;
    struct Frame {
        uint32_t node, next_child;
    };
    std::vector<Frame> stack;
    std::vector<uint32_t> path;
    for (uint32_t r = 0; r < D.root_count; ++r) {
        stack.assign(1, Frame{D.roots[r], 0});
        path.assign(1, D.roots[r]);
        bool entered = false;
        while (!stack.empty()) {
            Frame& f = stack.back();
            const vkgv_node& nd = D.nodes[f.node];
            if (!entered) {
                entered = true;
                if (++visits > (1u << 24)) {
                    err = "more than 2^24 node visits";
                    return VKGV_LIMIT_EXCEEDED;
                }
                if (nd.mesh_index != VKGV_INVALID_HANDLE) {
                    const uint32_t slot = (uint32_t)(P.chain_offsets.size() - 1);
                    P.chain_nodes.insert(P.chain_nodes.end(), path.begin(), path.end());
                    P.chain_offsets.push_back((uint32_t)P.chain_nodes.size());
                    for (uint32_t i = D.mesh_offsets[nd.mesh_index]; i < D.mesh_offsets[nd.mesh_index + 1]; ++i) {
                        const uint32_t prim = D.mesh_primitives[i];
                        const uint32_t count = D.primitive_meshlet_counts[prim];
                        if (!count) continue;
                        draws += count;
                        if (draws >= (1ull << 31)) {
                            err = "more than 2^31 meshlet draws";
                            return VKGV_LIMIT_EXCEEDED;
                        }
                        P.seg_info.push_back(make_uint2(prim, slot));
                        P.seg_first.push_back((uint32_t)draws);
                    }
                }
            }
            if (f.next_child < nd.child_count) {
                const uint32_t child = D.children[nd.first_child + f.next_child++];
                if (stack.size() >= VKGV_MAX_NODE_DEPTH) {
                    err = "node tree deeper than VKGV_MAX_NODE_DEPTH (or cyclic)";
                    return VKGV_LIMIT_EXCEEDED;
                }
                stack.push_back(Frame{child, 0});
                path.push_back(child);
                entered = false;
            } else {
                stack.pop_back();
                path.pop_back();
            }
        }
    }
    // first segment of every tile of kWorldTile draws
    const uint64_t tiles = (draws + kWorldTile - 1) / kWorldTile;
    P.tile_seg.resize(tiles);
    for (uint64_t t = 0, s = 0; t < tiles; ++t) {
        const uint64_t d = t * kWorldTile;
        while (s + 1 < P.seg_info.size() && P.seg_first[s + 1] <= d) ++s;
        P.tile_seg[t] = (uint32_t)s;
    }
    P.node_count = N;
    P.slot_count = (uint32_t)(P.chain_offsets.size() - 1);
    P.seg_count = (uint32_t)P.seg_info.size();
    P.draw_count = draws;
    return VKGV_OK;
}

}  // namespace vkgv
