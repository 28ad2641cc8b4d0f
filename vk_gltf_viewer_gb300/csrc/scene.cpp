// Host-side scene producers: procedural meshes, the meshletiser and the
// camera update.  These fill the renderer's own buffer layout (vkgv.h) the way
// the reference's importer does (src/vk_gltf_viewer/assets.cpp:288-430) and
// its camera does (src/vk_gltf_viewer/camera.cpp:38-84, 170-193).  They run
// once per scene on the host; nothing here is on the per-frame path.
#include "vkgv.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <utility>
#include <vector>

struct vkgv_mesh {
    std::vector<float> pos;      // 3 per vertex, the stored (dequantised) positions
    std::vector<float> normal;   // 3 per vertex
    std::vector<float> uv;       // 2 per vertex
    std::vector<float> rgba;     // 4 per vertex
    std::vector<uint32_t> idx;   // 3 per triangle
    std::vector<vkgv_vertex> verts;
    std::vector<vkgv_meshlet> meshlets;
    std::vector<vkgv_meshlet_cone> cones;
    std::vector<uint32_t> vtx_idx;
    std::vector<uint8_t> prim_idx;
    float aabb_ext[3] = {0, 0, 0};
    float aabb_ctr[3] = {0, 0, 0};
    float position_scale = 1.0f;
    int quantized_normals = 0;
};

namespace {

// ---------------------------------------------------------------- helpers

// IEEE binary32 -> binary16, round to nearest even (finite inputs in range).
uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    int32_t exp = int32_t((x >> 23) & 0xffu) - 127 + 15;
    uint32_t mant = x & 0x7fffffu;
    if (((x >> 23) & 0xffu) == 0xffu) return uint16_t(sign | 0x7c00u | (mant ? 0x200u : 0u));
    if (exp >= 31) return uint16_t(sign | 0x7c00u);
    if (exp <= 0) {
        if (exp < -10) return uint16_t(sign);
        mant |= 0x800000u;
        uint32_t shift = uint32_t(14 - exp);
        uint32_t half = mant >> shift;
        uint32_t rem = mant & ((1u << shift) - 1u);
        uint32_t mid = 1u << (shift - 1u);
        if (rem > mid || (rem == mid && (half & 1u))) ++half;
        return uint16_t(sign | half);
    }
    uint32_t half = sign | (uint32_t(exp) << 10) | (mant >> 13);
    uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ++half;
    return uint16_t(half);
}

// splitmix64: seeded, platform-independent random stream.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    // uniform in [-1, 1)
    double sym() { return double(next() >> 11) * (2.0 / 9007199254740992.0) - 1.0; }
};

// Periodic 2D value noise on a gx x gy lattice with smoothstep blending,
// returning values in [-1, 1].
struct ValueNoise2 {
    int gx, gy;
    std::vector<double> v;
    ValueNoise2(int gx_, int gy_, uint64_t seed) : gx(gx_), gy(gy_), v(size_t(gx_) * gy_) {
        Rng r(seed);
        for (auto& x : v) x = r.sym();
    }
    double at(double s, double t) const {  // s, t in [0, 1], periodic
        double x = s * gx, y = t * gy;
        int x0 = int(std::floor(x)), y0 = int(std::floor(y));
        double fx = x - x0, fy = y - y0;
        fx = fx * fx * (3 - 2 * fx);
        fy = fy * fy * (3 - 2 * fy);
        auto g = [&](int i, int j) {
            i = ((i % gx) + gx) % gx;
            j = ((j % gy) + gy) % gy;
            return v[size_t(j) * gx + i];
        };
        double a = g(x0, y0) + (g(x0 + 1, y0) - g(x0, y0)) * fx;
        double b = g(x0, y0 + 1) + (g(x0 + 1, y0 + 1) - g(x0, y0 + 1)) * fx;
        return a + (b - a) * fy;
    }
};

// 3D value noise on the integer lattice of a scaled point.
struct ValueNoise3 {
    uint64_t seed;
    explicit ValueNoise3(uint64_t s) : seed(s) {}
    double lattice(int64_t i, int64_t j, int64_t k) const {
        Rng r(seed ^ (uint64_t(i) * 0x8da6b343ull) ^ (uint64_t(j) * 0xd8163841ull) ^
              (uint64_t(k) * 0xcb1ab31full));
        return r.sym();
    }
    double at(double x, double y, double z) const {
        int64_t x0 = int64_t(std::floor(x)), y0 = int64_t(std::floor(y)), z0 = int64_t(std::floor(z));
        double fx = x - x0, fy = y - y0, fz = z - z0;
        fx = fx * fx * (3 - 2 * fx);
        fy = fy * fy * (3 - 2 * fy);
        fz = fz * fz * (3 - 2 * fz);
        double c[2][2][2];
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(x0 + a, y0 + b, z0 + d);
        double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * fx;
        double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * fx;
        double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * fx;
        double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * fx;
        double y0v = x00 + (x10 - x00) * fy;
        double y1v = x01 + (x11 - x01) * fy;
        return y0v + (y1v - y0v) * fz;
    }
};

void compute_aabb(vkgv_mesh& m) {
    size_t nv = m.pos.size() / 3;
    if (nv == 0) return;
    float mn[3] = {m.pos[0], m.pos[1], m.pos[2]}, mx[3] = {m.pos[0], m.pos[1], m.pos[2]};
    for (size_t i = 1; i < nv; ++i)
        for (int c = 0; c < 3; ++c) {
            mn[c] = std::min(mn[c], m.pos[3 * i + c]);
            mx[c] = std::max(mx[c], m.pos[3 * i + c]);
        }
    // Accessor min/max -> centre and extents (assets.cpp:301-306).
    for (int c = 0; c < 3; ++c) {
        m.aabb_ctr[c] = (mn[c] + mx[c]) / 2.f;
        m.aabb_ext[c] = mx[c] - m.aabb_ctr[c];
    }
}

uint8_t encode_normal(float n) {
    // int8-normalised value q in [-127, 127] stored biased as q + 127, so
    // that the reference unpack (n / 127 - 1) returns q / 127.
    float c = std::max(-1.f, std::min(1.f, n));
    int q = int(std::lrint(c * 127.f));
    return uint8_t(q + 127);
}

void fill_vertex_stream(vkgv_mesh& m) {
    size_t nv = m.pos.size() / 3;
    m.verts.assign(nv, vkgv_vertex{});
    for (size_t i = 0; i < nv; ++i) {
        vkgv_vertex& v = m.verts[i];
        for (int c = 0; c < 3; ++c) v.position[c] = m.pos[3 * i + c];
        for (int c = 0; c < 4; ++c) {
            float x = m.rgba.empty() ? 1.f : m.rgba[4 * i + c];
            x = std::max(0.f, std::min(1.f, x));
            v.color[c] = uint8_t(std::lrint(x * 255.f));
        }
        for (int c = 0; c < 3; ++c) v.normal[c] = m.normal.empty() ? 127 : encode_normal(m.normal[3 * i + c]);
        v._pad = 0;
        for (int c = 0; c < 2; ++c) v.uv[c] = float_to_half(m.uv.empty() ? 0.f : m.uv[2 * i + c]);
    }
}

// Makes every triangle wind counter-clockwise around the outward normal
// given by `outward` (a direction per triangle).
template <class F>
void orient_triangles(vkgv_mesh& m, F outward) {
    size_t nt = m.idx.size() / 3;
    for (size_t t = 0; t < nt; ++t) {
        const float* a = &m.pos[3 * m.idx[3 * t]];
        const float* b = &m.pos[3 * m.idx[3 * t + 1]];
        const float* c = &m.pos[3 * m.idx[3 * t + 2]];
        double e1[3], e2[3], n[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = double(b[k]) - a[k];
            e2[k] = double(c[k]) - a[k];
        }
        n[0] = e1[1] * e2[2] - e1[2] * e2[1];
        n[1] = e1[2] * e2[0] - e1[0] * e2[2];
        n[2] = e1[0] * e2[1] - e1[1] * e2[0];
        std::array<double, 3> o = outward(t);
        if (n[0] * o[0] + n[1] * o[1] + n[2] * o[2] < 0) std::swap(m.idx[3 * t + 1], m.idx[3 * t + 2]);
    }
}

}  // namespace

// ------------------------------------------------------------- icosphere

extern "C" vkgv_mesh* vkgv_mesh_icosphere(uint32_t level) {
    if (level > 10) return nullptr;
    vkgv_mesh* m = new (std::nothrow) vkgv_mesh();
    if (!m) return nullptr;
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> p = {
        {-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
        {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto& v : p) {
        double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (auto& c : v) c /= l;
    }
    // The 20 faces of the icosahedron over the 12 vertices above.
    std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11,
                               1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
                               3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9,
                               4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (uint32_t l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            std::array<double, 3> v;
            for (int c = 0; c < 3; ++c) v[c] = (p[a][c] + p[b][c]) * 0.5;
            double len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            for (auto& c : v) c /= len;
            p.push_back(v);
            uint32_t id = uint32_t(p.size() - 1);
            mid.emplace(key, id);
            return id;
        };
        std::vector<uint32_t> g;
        g.reserve(f.size() * 4);
        // Children of face i stay contiguous, so faces keep a spatially
        // coherent (hierarchical) order for the meshletiser.
        for (size_t i = 0; i < f.size(); i += 3) {
            uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            g.insert(g.end(), tri, tri + 12);
        }
        f.swap(g);
    }
    m->pos.resize(p.size() * 3);
    m->normal.resize(p.size() * 3);
    m->uv.resize(p.size() * 2);
    const double pi = 3.14159265358979323846;
    for (size_t i = 0; i < p.size(); ++i) {
        for (int c = 0; c < 3; ++c) {
            m->pos[3 * i + c] = float(p[i][c]);
            m->normal[3 * i + c] = float(p[i][c]);
        }
        // Equirectangular UV.
        m->uv[2 * i] = float(0.5 + std::atan2(p[i][2], p[i][0]) / (2 * pi));
        m->uv[2 * i + 1] = float(std::acos(std::max(-1.0, std::min(1.0, p[i][1]))) / pi);
    }
    m->idx = f;
    orient_triangles(*m, [&](size_t tri) {
        std::array<double, 3> o{0, 0, 0};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) o[c] += p[m->idx[3 * tri + k]][c];
        return o;
    });
    compute_aabb(*m);
    fill_vertex_stream(*m);
    return m;
}

extern "C" int vkgv_mesh_displace(vkgv_mesh* m, float amp, uint64_t seed) {
    if (!m) return VKGV_INVALID_ARG;
    ValueNoise3 noise(seed);
    size_t nv = m->pos.size() / 3;
    for (size_t i = 0; i < nv; ++i) {
        double x = m->pos[3 * i], y = m->pos[3 * i + 1], z = m->pos[3 * i + 2];
        double l = std::sqrt(x * x + y * y + z * z);
        if (l == 0) continue;
        double d = amp * noise.at(x * 4 + 11.5, y * 4 + 7.25, z * 4 + 3.125);
        double s = (l + d) / l;
        m->pos[3 * i] = float(x * s);
        m->pos[3 * i + 1] = float(y * s);
        m->pos[3 * i + 2] = float(z * s);
    }
    compute_aabb(*m);
    fill_vertex_stream(*m);
    m->meshlets.clear();
    m->cones.clear();
    m->vtx_idx.clear();
    m->prim_idx.clear();
    return VKGV_OK;
}

// ----------------------------------------------------------------- torus

extern "C" vkgv_mesh* vkgv_mesh_torus(float R, float r, uint32_t seg_major, uint32_t seg_minor,
                                      float noise_amp, uint64_t seed, int32_t quantize) {
    if (seg_major < 3 || seg_minor < 3 || seg_major > 4096 || seg_minor > 4096) return nullptr;
    vkgv_mesh* m = new (std::nothrow) vkgv_mesh();
    if (!m) return nullptr;
    const double pi = 3.14159265358979323846;
    // Seam-split grid so UVs stay continuous: (seg_major+1) x (seg_minor+1).
    const uint32_t nu = seg_major + 1, nvv = seg_minor + 1;
    ValueNoise2 noise(20, 10, seed);
    std::vector<double> P(size_t(nu) * nvv * 3), N(size_t(nu) * nvv * 3);
    for (uint32_t j = 0; j < nvv; ++j) {
        for (uint32_t i = 0; i < nu; ++i) {
            double s = double(i) / seg_major, t = double(j) / seg_minor;
            double u = 2 * pi * s, v = 2 * pi * t;
            double n[3] = {std::cos(v) * std::cos(u), std::sin(v), std::cos(v) * std::sin(u)};
            double d = r + noise_amp * noise.at(s, t);
            size_t k = (size_t(j) * nu + i) * 3;
            P[k] = R * std::cos(u) + d * n[0];
            P[k + 1] = d * n[1];
            P[k + 2] = R * std::sin(u) + d * n[2];
            for (int c = 0; c < 3; ++c) N[k + c] = n[c];
        }
    }
    size_t nv = size_t(nu) * nvv;
    m->pos.resize(nv * 3);
    m->normal.resize(nv * 3);
    m->uv.resize(nv * 2);
    double maxabs = 0;
    for (double x : P) maxabs = std::max(maxabs, std::fabs(x));
    if (quantize) {
        // KHR_mesh_quantization: SHORT normalised positions q / 32767 with the
        // dequantisation scale left to the node matrix; BYTE normalised normals.
        double scale = std::ceil(maxabs * 64.0) / 64.0;
        m->position_scale = float(scale);
        for (size_t k = 0; k < nv * 3; ++k) {
            long q = std::lrint(P[k] / scale * 32767.0);
            q = std::max(-32767L, std::min(32767L, q));
            m->pos[k] = std::max(float(q) / 32767.0f, -1.0f);
            long qn = std::lrint(N[k] * 127.0);
            m->normal[k] = std::max(float(qn) / 127.0f, -1.0f);
        }
        m->quantized_normals = 1;
    } else {
        for (size_t k = 0; k < nv * 3; ++k) {
            m->pos[k] = float(P[k]);
            m->normal[k] = float(N[k]);
        }
    }
    for (uint32_t j = 0; j < nvv; ++j)
        for (uint32_t i = 0; i < nu; ++i) {
            m->uv[2 * (size_t(j) * nu + i)] = float(double(i) / seg_major);
            m->uv[2 * (size_t(j) * nu + i) + 1] = float(double(j) / seg_minor);
        }
    // Emit quads in 7 x 7 blocks so consecutive triangles share vertices.
    const uint32_t B = 7;
    for (uint32_t bj = 0; bj < seg_minor; bj += B)
        for (uint32_t bi = 0; bi < seg_major; bi += B)
            for (uint32_t j = bj; j < std::min(bj + B, seg_minor); ++j)
                for (uint32_t i = bi; i < std::min(bi + B, seg_major); ++i) {
                    uint32_t a = j * nu + i, b = j * nu + i + 1, c = (j + 1) * nu + i + 1, d = (j + 1) * nu + i;
                    uint32_t q[6] = {a, b, c, a, c, d};
                    m->idx.insert(m->idx.end(), q, q + 6);
                }
    orient_triangles(*m, [&](size_t tri) {
        std::array<double, 3> o{0, 0, 0};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) o[c] += N[size_t(m->idx[3 * tri + k]) * 3 + c];
        return o;
    });
    compute_aabb(*m);
    fill_vertex_stream(*m);
    return m;
}

extern "C" vkgv_mesh* vkgv_mesh_from_arrays(const float* positions, uint32_t vertex_count,
                                            const uint32_t* indices, uint32_t triangle_count) {
    if (!positions || !indices || vertex_count == 0) return nullptr;
    for (uint64_t i = 0; i < uint64_t(triangle_count) * 3; ++i)
        if (indices[i] >= vertex_count) return nullptr;
    vkgv_mesh* m = new (std::nothrow) vkgv_mesh();
    if (!m) return nullptr;
    m->pos.assign(positions, positions + size_t(vertex_count) * 3);
    m->idx.assign(indices, indices + size_t(triangle_count) * 3);
    compute_aabb(*m);
    fill_vertex_stream(*m);
    return m;
}

extern "C" int vkgv_mesh_set_attributes(vkgv_mesh* m, const float* rgba, const float* uv) {
    if (!m) return VKGV_INVALID_ARG;
    size_t nv = m->pos.size() / 3;
    if (rgba) m->rgba.assign(rgba, rgba + nv * 4);
    if (uv) m->uv.assign(uv, uv + nv * 2);
    fill_vertex_stream(*m);
    return VKGV_OK;
}

// ------------------------------------------------------------ meshletiser

namespace {

// Normal cone of a meshlet (object space), rounded so that it stays a
// bound in fp32: cutoff rounded down, radius rounded up.  A meshlet with a
// degenerate triangle or a cone wider than ~87 degrees gets cutoff -1
// (never culled).
vkgv_meshlet_cone meshlet_cone(const vkgv_mesh& m, const std::vector<uint32_t>& tris,
                               const std::vector<uint32_t>& verts, const float* center) {
    vkgv_meshlet_cone cone{};
    for (int c = 0; c < 3; ++c) cone.center[c] = center[c];
    double r2 = 0;
    for (uint32_t v : verts) {
        double d2 = 0;
        for (int c = 0; c < 3; ++c) {
            double e = double(m.pos[3 * size_t(v) + c]) - double(center[c]);
            d2 += e * e;
        }
        r2 = std::max(r2, d2);
    }
    double r = std::sqrt(r2) * (1.0 + 1e-6) + 1e-7;
    cone.radius = std::nextafter(float(r), INFINITY);
    cone.cutoff = -1.0f;
    std::vector<std::array<double, 3>> normals;
    double sum[3] = {0, 0, 0};
    for (uint32_t t : tris) {
        const float* a = &m.pos[3 * size_t(m.idx[3 * t])];
        const float* b = &m.pos[3 * size_t(m.idx[3 * t + 1])];
        const float* c = &m.pos[3 * size_t(m.idx[3 * t + 2])];
        double e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = double(b[k]) - a[k];
            e2[k] = double(c[k]) - a[k];
        }
        std::array<double, 3> n = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                   e1[0] * e2[1] - e1[1] * e2[0]};
        double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (!(len > 1e-30)) return cone;  // degenerate triangle: no cone
        for (double& x : n) x /= len;
        normals.push_back(n);
        for (int k = 0; k < 3; ++k) sum[k] += n[k];
    }
    double sl = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
    if (!(sl > 1e-12)) return cone;
    double axis[3] = {sum[0] / sl, sum[1] / sl, sum[2] / sl};
    double cmin = 1.0;
    for (auto& n : normals) cmin = std::min(cmin, n[0] * axis[0] + n[1] * axis[1] + n[2] * axis[2]);
    if (!(cmin > 0.05)) return cone;
    for (int k = 0; k < 3; ++k) cone.axis[k] = float(axis[k]);
    // The stored axis is the rounded one: recompute the bound against it.
    double cmin_f = 1.0;
    double fa[3] = {cone.axis[0], cone.axis[1], cone.axis[2]};
    double fal = std::sqrt(fa[0] * fa[0] + fa[1] * fa[1] + fa[2] * fa[2]);
    for (auto& n : normals) cmin_f = std::min(cmin_f, (n[0] * fa[0] + n[1] * fa[1] + n[2] * fa[2]) / fal);
    cmin_f -= 1e-6;
    if (!(cmin_f > 0.05)) return cone;
    cone.cutoff = std::nextafter(float(cmin_f), -INFINITY);
    return cone;
}

}  // namespace

// Greedy, adjacency-driven meshletiser.  Like meshopt_buildMeshlets with
// coneWeight 0 (assets.cpp:323-341) it grows one meshlet at a time under the
// vertex and triangle limits; it prefers the adjacent triangle that adds the
// fewest new vertices and starts a new meshlet when none fits.  The exact
// partition differs from meshoptimizer's (which is not vendored); the layout
// and limits are the same.
extern "C" int vkgv_mesh_build_meshlets(vkgv_mesh* m, uint32_t max_v, uint32_t max_t) {
    if (!m || max_v < 3 || max_v > 255 || max_t < 1 || max_t > 255) return VKGV_INVALID_ARG;
    const size_t nv = m->pos.size() / 3, nt = m->idx.size() / 3;
    m->meshlets.clear();
    m->cones.clear();
    m->vtx_idx.clear();
    m->prim_idx.clear();
    // vertex -> triangles adjacency (CSR)
    std::vector<uint32_t> off(nv + 1, 0), adj(nt * 3);
    for (size_t i = 0; i < nt * 3; ++i) off[m->idx[i] + 1]++;
    for (size_t v = 0; v < nv; ++v) off[v + 1] += off[v];
    {
        std::vector<uint32_t> fill(off.begin(), off.end() - 1);
        for (size_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) adj[fill[m->idx[3 * t + k]]++] = uint32_t(t);
    }
    std::vector<uint8_t> used(nt, 0);
    std::vector<int32_t> local(nv, -1);
    std::vector<uint32_t> stamp(nt, 0);
    uint32_t cur_stamp = 0;
    size_t seed = 0, remaining = nt;
    std::vector<uint32_t> mverts, mtris, cand;
    while (remaining > 0) {
        while (used[seed]) ++seed;
        ++cur_stamp;
        mverts.clear();
        mtris.clear();
        cand.clear();
        auto add_tri = [&](uint32_t t) {
            used[t] = 1;
            --remaining;
            mtris.push_back(t);
            for (int k = 0; k < 3; ++k) {
                uint32_t v = m->idx[3 * t + k];
                if (local[v] < 0) {
                    local[v] = int32_t(mverts.size());
                    mverts.push_back(v);
                    for (uint32_t e = off[v]; e < off[v + 1]; ++e) {
                        uint32_t u = adj[e];
                        if (!used[u] && stamp[u] != cur_stamp) {
                            stamp[u] = cur_stamp;
                            cand.push_back(u);
                        }
                    }
                }
            }
        };
        add_tri(uint32_t(seed));
        while (mtris.size() < max_t) {
            int best = -1, best_new = 4;
            size_t w = 0;
            for (size_t i = 0; i < cand.size(); ++i) {
                uint32_t u = cand[i];
                if (used[u]) continue;
                cand[w++] = u;
                int nn = 0;
                for (int k = 0; k < 3; ++k) nn += local[m->idx[3 * u + k]] < 0;
                if (nn < best_new) {
                    best_new = nn;
                    best = int(u);
                }
            }
            cand.resize(w);
            if (best < 0 || mverts.size() + size_t(best_new) > max_v) break;
            add_tri(uint32_t(best));
        }
        vkgv_meshlet ml{};
        ml.vertex_offset = uint32_t(m->vtx_idx.size());
        ml.triangle_offset = uint32_t(m->prim_idx.size());
        ml.vertex_count = uint8_t(mverts.size());
        ml.triangle_count = uint8_t(mtris.size());
        m->vtx_idx.insert(m->vtx_idx.end(), mverts.begin(), mverts.end());
        for (uint32_t t : mtris)
            for (int k = 0; k < 3; ++k) m->prim_idx.push_back(uint8_t(local[m->idx[3 * t + k]]));
        while (m->prim_idx.size() & 3u) m->prim_idx.push_back(0);  // 4-byte aligned blocks
        // Meshlet AABB from its vertices (assets.cpp:348-372).
        float mn[3], mx[3];
        for (int c = 0; c < 3; ++c) mn[c] = mx[c] = m->pos[3 * size_t(mverts[0]) + c];
        for (size_t i = 1; i < mverts.size(); ++i)
            for (int c = 0; c < 3; ++c) {
                float x = m->pos[3 * size_t(mverts[i]) + c];
                mn[c] = std::min(mn[c], x);
                mx[c] = std::max(mx[c], x);
            }
        for (int c = 0; c < 3; ++c) {
            float ctr = (mn[c] + mx[c]) * 0.5f;
            ml.aabb_center[c] = ctr;
            ml.aabb_extents[c] = mx[c] - ctr;
        }
        m->meshlets.push_back(ml);
        m->cones.push_back(meshlet_cone(*m, mtris, mverts, ml.aabb_center));
        for (uint32_t v : mverts) local[v] = -1;
    }
    return VKGV_OK;
}

extern "C" int vkgv_mesh_get_info(const vkgv_mesh* m, vkgv_mesh_info* out) {
    if (!m || !out) return VKGV_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->vertex_count = uint32_t(m->pos.size() / 3);
    out->triangle_count = uint32_t(m->idx.size() / 3);
    out->meshlet_count = uint32_t(m->meshlets.size());
    out->vertex_index_count = uint32_t(m->vtx_idx.size());
    out->primitive_index_bytes = uint32_t(m->prim_idx.size());
    out->position_scale = m->position_scale;
    out->vertices = m->verts.data();
    out->positions = m->pos.data();
    out->uvs = m->uv.empty() ? nullptr : m->uv.data();
    out->indices = m->idx.data();
    out->meshlets = m->meshlets.empty() ? nullptr : m->meshlets.data();
    out->vertex_indices = m->vtx_idx.empty() ? nullptr : m->vtx_idx.data();
    out->primitive_indices = m->prim_idx.empty() ? nullptr : m->prim_idx.data();
    out->cones = m->cones.empty() ? nullptr : m->cones.data();
    for (int c = 0; c < 3; ++c) {
        out->aabb_extents[c] = m->aabb_ext[c];
        out->aabb_center[c] = m->aabb_ctr[c];
    }
    return VKGV_OK;
}

extern "C" void vkgv_mesh_free(vkgv_mesh* m) { delete m; }

// ---------------------------------------------------------------- camera

namespace {
using M4 = std::array<float, 16>;  // column-major, m[c*4 + r]

M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float s = 0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = s;
        }
    return r;
}
}  // namespace

extern "C" int vkgv_frustum_planes(const float vp[16], float out[24]) {
    if (!vp || !out) return VKGV_INVALID_ARG;
    // Plane k = row 3 +/- row {0, 1, 2} of VP (camera.cpp:70-84), normalised
    // by the length of its xyz, with w negated.
    for (int k = 0; k < 6; ++k) {
        int row = k / 2;
        float sgn = (k & 1) ? -1.f : 1.f;
        float pl[4];
        for (int i = 0; i < 4; ++i) pl[i] = vp[i * 4 + 3] + sgn * vp[i * 4 + row];
        float len = std::sqrt(pl[0] * pl[0] + pl[1] * pl[1] + pl[2] * pl[2]);
        if (!(len > 0)) return VKGV_INVALID_ARG;
        for (int i = 0; i < 4; ++i) pl[i] /= len;
        pl[3] = -pl[3];
        for (int i = 0; i < 4; ++i) out[k * 4 + i] = pl[i];
    }
    return VKGV_OK;
}

extern "C" int vkgv_camera_update(vkgv_camera* cam, const float eye[3], const float target[3],
                                  const float up[3], float fovy, float aspect, float znear, float zfar) {
    if (!cam || !eye || !target || !up) return VKGV_INVALID_ARG;
    if (!(fovy > 0 && fovy < 3.14159f) || !(aspect > 0) || !(znear > 0) || !(zfar > znear))
        return VKGV_INVALID_ARG;
    // Right-handed look-at view matrix.
    float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
    float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0)) return VKGV_INVALID_ARG;
    for (float& x : f) x /= fl;
    float s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    float sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (!(sl > 0)) return VKGV_INVALID_ARG;  // up parallel to the view direction
    for (float& x : s) x /= sl;
    float u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    M4 view{};
    for (int i = 0; i < 3; ++i) {
        view[i * 4 + 0] = s[i];
        view[i * 4 + 1] = u[i];
        view[i * 4 + 2] = -f[i];
    }
    view[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    view[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    view[14] = (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2]);
    view[15] = 1.f;
    // Right-handed perspective with a [0, 1] depth range, then the Y flip
    // (camera.cpp:177-178).
    const float th = std::tan(fovy / 2.f);
    M4 proj{};
    proj[0] = 1.f / (aspect * th);
    proj[5] = -(1.f / th);
    proj[10] = zfar / (znear - zfar);
    proj[11] = -1.f;
    proj[14] = -(zfar * znear) / (zfar - znear);
    // Reverse-Z: z' = w - z (camera.cpp:38-48).
    M4 rz{};
    rz[0] = 1.f;
    rz[5] = 1.f;
    rz[10] = -1.f;
    rz[14] = 1.f;
    rz[15] = 1.f;
    M4 vp = mul(mul(rz, proj), view);
    // Shift current -> prev, then write current (camera.cpp:180-193).
    std::memcpy(cam->prev_view_projection, cam->view_projection, 64);
    std::memcpy(cam->prev_occlusion_view_projection, cam->occlusion_view_projection, 64);
    std::memcpy(cam->view_projection, vp.data(), 64);
    std::memcpy(cam->occlusion_view_projection, vp.data(), 64);
    return vkgv_frustum_planes(vp.data(), &cam->frustum[0][0]);
}

extern "C" int vkgv_pyramid_layout(uint32_t w, uint32_t h, uint32_t* out_levels, uint64_t* out_floats) {
    if (!out_levels || !out_floats) return VKGV_INVALID_ARG;
    if (w == 0 || h == 0 || w > VKGV_MAX_VIEW_DIM || h > VKGV_MAX_VIEW_DIM) return VKGV_INVALID_ARG;
    uint32_t mx = std::max(w, h);
    uint32_t levels = 0;
    while ((2u << levels) <= mx) ++levels;  // floor(log2(max(W, H))) (application.cpp:472-473)
    uint64_t total = 0;
    for (uint32_t k = 0; k < levels; ++k) {
        uint64_t mw = std::max(1u, (w >> 1) >> k), mh = std::max(1u, (h >> 1) >> k);
        total += mw * mh;
    }
    *out_levels = levels;
    *out_floats = total;
    return VKGV_OK;
}

extern "C" const char* vkgv_version(void) { return "vkgv 0.1.0 (sm_103a)"; }
