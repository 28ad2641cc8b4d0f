/*
 * scene.c — CPU restatement of the host scene producers (procedural meshes,
 * the greedy meshletiser with normal cones, the camera update).  TEST
 * INFRASTRUCTURE ONLY: it lets the benchmark's reference arm and the tests
 * build the C1/C2 scenes and camera buffers without loading the product
 * library.  A CPU test checks that every buffer it produces is byte-identical
 * to the product's own producers.
 *
 * Reference anchors: meshlet layout and per-meshlet AABB from its vertices
 * (src/vk_gltf_viewer/assets.cpp:323-372, shaders/mesh_common.h.glsl:49-58),
 * accessor min/max -> centre/extents (assets.cpp:301-306), camera matrices
 * (src/vk_gltf_viewer/camera.cpp:38-48, 170-193) and frustum planes
 * (camera.cpp:70-84).  The mesh generators themselves are synthetic inputs
 * with no reference counterpart.
 *
 * Built with -ffp-contract=off and no fast-math, like the product's host
 * code, so the float results round identically.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct orc_mesh {
    float* pos;     /* 3 per vertex */
    float* normal;  /* 3 per vertex, or NULL */
    float* uv;      /* 2 per vertex, or NULL */
    uint32_t* idx;  /* 3 per triangle */
    uint32_t nv, nt;
    orc_vertex* verts;
    orc_meshlet* meshlets;
    orc_cone* cones;
    uint32_t* vtx_idx;
    uint8_t* prim_idx;
    uint32_t meshlet_count, vtx_idx_count, prim_idx_bytes;
    float aabb_ext[3], aabb_ctr[3];
    float position_scale;
} orc_mesh;

/* What orc_mesh_get_info returns (pointers into the mesh). */
typedef struct orc_mesh_info {
    uint32_t vertex_count, triangle_count, meshlet_count, vertex_index_count, primitive_index_bytes;
    float position_scale;
    const orc_vertex* vertices;
    const float* positions;
    const float* uvs;
    const uint32_t* indices;
    const orc_meshlet* meshlets;
    const uint32_t* vertex_indices;
    const uint8_t* primitive_indices;
    const orc_cone* cones;
    float aabb_extents[3], aabb_center[3];
} orc_mesh_info;

/* ---------------------------------------------------------------- helpers */

static uint16_t half_rn(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    int32_t e = (int32_t)((x >> 23) & 0xffu) - 127 + 15;
    uint32_t mant = x & 0x7fffffu;
    if (((x >> 23) & 0xffu) == 0xffu) return (uint16_t)(sign | 0x7c00u | (mant ? 0x200u : 0u));
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - e);
        uint32_t h = mant >> shift, rem = mant & ((1u << shift) - 1u), mid = 1u << (shift - 1u);
        if (rem > mid || (rem == mid && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = sign | ((uint32_t)e << 10) | (mant >> 13);
    uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)h;
}

/* splitmix64 */
static uint64_t rng_next(uint64_t* s) {
    uint64_t z = (*s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double rng_sym(uint64_t* s) { return (double)(rng_next(s) >> 11) * (2.0 / 9007199254740992.0) - 1.0; }

static double smooth(double f) { return f * f * (3 - 2 * f); }

/* periodic 2D value noise on a gx x gy lattice */
static double noise2(const double* lat, int gx, int gy, double s, double t) {
    double x = s * gx, y = t * gy;
    int x0 = (int)floor(x), y0 = (int)floor(y);
    double fx = smooth(x - x0), fy = smooth(y - y0);
#define G(i, j) lat[(size_t)(((((j) % gy) + gy) % gy)) * gx + (size_t)((((i) % gx) + gx) % gx)]
    double a = G(x0, y0) + (G(x0 + 1, y0) - G(x0, y0)) * fx;
    double b = G(x0, y0 + 1) + (G(x0 + 1, y0 + 1) - G(x0, y0 + 1)) * fx;
#undef G
    return a + (b - a) * fy;
}

static double lattice3(uint64_t seed, int64_t i, int64_t j, int64_t k) {
    uint64_t s = seed ^ ((uint64_t)i * 0x8da6b343ull) ^ ((uint64_t)j * 0xd8163841ull) ^ ((uint64_t)k * 0xcb1ab31full);
    return rng_sym(&s);
}

static double noise3(uint64_t seed, double x, double y, double z) {
    int64_t x0 = (int64_t)floor(x), y0 = (int64_t)floor(y), z0 = (int64_t)floor(z);
    double fx = smooth(x - x0), fy = smooth(y - y0), fz = smooth(z - z0);
    double c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice3(seed, x0 + a, y0 + b, z0 + d);
    double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * fx;
    double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * fx;
    double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * fx;
    double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * fx;
    double y0v = x00 + (x10 - x00) * fy;
    double y1v = x01 + (x11 - x01) * fy;
    return y0v + (y1v - y0v) * fz;
}

static float fminf_(float a, float b) { return b < a ? b : a; }
static float fmaxf_(float a, float b) { return a < b ? b : a; }

/* accessor min/max -> centre and extents (assets.cpp:301-306) */
static void compute_aabb(orc_mesh* m) {
    if (m->nv == 0) return;
    float mn[3] = {m->pos[0], m->pos[1], m->pos[2]}, mx[3] = {m->pos[0], m->pos[1], m->pos[2]};
    for (uint32_t i = 1; i < m->nv; ++i)
        for (int c = 0; c < 3; ++c) {
            mn[c] = fminf_(mn[c], m->pos[3 * (size_t)i + c]);
            mx[c] = fmaxf_(mx[c], m->pos[3 * (size_t)i + c]);
        }
    for (int c = 0; c < 3; ++c) {
        m->aabb_ctr[c] = (mn[c] + mx[c]) / 2.f;
        m->aabb_ext[c] = mx[c] - m->aabb_ctr[c];
    }
}

static uint8_t encode_normal(float n) {
    float c = fmaxf_(-1.f, fminf_(1.f, n));
    int q = (int)lrintf(c * 127.f);
    return (uint8_t)(q + 127);
}

static void fill_vertex_stream(orc_mesh* m) {
    free(m->verts);
    m->verts = (orc_vertex*)calloc(m->nv ? m->nv : 1, sizeof(orc_vertex));
    for (uint32_t i = 0; i < m->nv; ++i) {
        orc_vertex* v = &m->verts[i];
        for (int c = 0; c < 3; ++c) v->position[c] = m->pos[3 * (size_t)i + c];
        for (int c = 0; c < 4; ++c) v->color[c] = (uint8_t)lrintf(1.f * 255.f);
        for (int c = 0; c < 3; ++c) v->normal[c] = m->normal ? encode_normal(m->normal[3 * (size_t)i + c]) : 127;
        v->pad_ = 0;
        for (int c = 0; c < 2; ++c) v->uv[c] = half_rn(m->uv ? m->uv[2 * (size_t)i + c] : 0.f);
    }
}

/* every triangle wound counter-clockwise around `out` (one direction per
 * triangle, 3 doubles each) */
static void orient(orc_mesh* m, const double* out) {
    for (uint32_t t = 0; t < m->nt; ++t) {
        const float* a = &m->pos[3 * (size_t)m->idx[3 * t]];
        const float* b = &m->pos[3 * (size_t)m->idx[3 * t + 1]];
        const float* c = &m->pos[3 * (size_t)m->idx[3 * t + 2]];
        double e1[3], e2[3], n[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = (double)b[k] - a[k];
            e2[k] = (double)c[k] - a[k];
        }
        n[0] = e1[1] * e2[2] - e1[2] * e2[1];
        n[1] = e1[2] * e2[0] - e1[0] * e2[2];
        n[2] = e1[0] * e2[1] - e1[1] * e2[0];
        const double* o = out + 3 * (size_t)t;
        if (n[0] * o[0] + n[1] * o[1] + n[2] * o[2] < 0) {
            uint32_t tmp = m->idx[3 * t + 1];
            m->idx[3 * t + 1] = m->idx[3 * t + 2];
            m->idx[3 * t + 2] = tmp;
        }
    }
}

static void clear_meshlets(orc_mesh* m) {
    free(m->meshlets);
    free(m->cones);
    free(m->vtx_idx);
    free(m->prim_idx);
    m->meshlets = NULL;
    m->cones = NULL;
    m->vtx_idx = NULL;
    m->prim_idx = NULL;
    m->meshlet_count = m->vtx_idx_count = m->prim_idx_bytes = 0;
}

void orc_mesh_free(orc_mesh* m) {
    if (!m) return;
    clear_meshlets(m);
    free(m->pos);
    free(m->normal);
    free(m->uv);
    free(m->idx);
    free(m->verts);
    free(m);
}

/* ------------------------------------------------------------- icosphere */

/* open-addressing map (edge key -> midpoint vertex) */
typedef struct {
    uint64_t* keys;
    uint32_t* vals;
    size_t cap;
} edge_map;

static uint32_t edge_mid(edge_map* e, double (**p)[3], uint32_t* np, size_t* pcap, uint32_t a, uint32_t b) {
    uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    uint64_t key = ((uint64_t)lo << 32) | hi;
    size_t h = (size_t)((key * 0x9e3779b97f4a7c15ull) >> 20) & (e->cap - 1);
    while (e->keys[h] != UINT64_MAX) {
        if (e->keys[h] == key) return e->vals[h];
        h = (h + 1) & (e->cap - 1);
    }
    double v[3];
    double (*P)[3] = *p;
    for (int c = 0; c < 3; ++c) v[c] = (P[a][c] + P[b][c]) * 0.5;
    double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) v[c] /= len;
    if (*np == *pcap) {
        *pcap *= 2;
        *p = (double (*)[3])realloc(*p, *pcap * sizeof(double[3]));
    }
    for (int c = 0; c < 3; ++c) (*p)[*np][c] = v[c];
    uint32_t id = (*np)++;
    e->keys[h] = key;
    e->vals[h] = id;
    return id;
}

orc_mesh* orc_mesh_icosphere(uint32_t level) {
    if (level > 10) return NULL;
    orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
    m->position_scale = 1.0f;
    const double t = (1.0 + sqrt(5.0)) / 2.0;
    const double base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                                {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    size_t pcap = 16;
    uint32_t np = 12;
    double (*p)[3] = (double (*)[3])malloc(pcap * sizeof(double[3]));
    for (int i = 0; i < 12; ++i) {
        double l = sqrt(base[i][0] * base[i][0] + base[i][1] * base[i][1] + base[i][2] * base[i][2]);
        for (int c = 0; c < 3; ++c) p[i][c] = base[i][c] / l;
    }
    static const uint32_t faces[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                                       11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                                       3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    size_t nf = 60;
    uint32_t* f = (uint32_t*)malloc(nf * sizeof(uint32_t));
    memcpy(f, faces, sizeof(faces));
    for (uint32_t l = 0; l < level; ++l) {
        edge_map e;
        e.cap = 1;
        while (e.cap < nf * 2) e.cap <<= 1;
        e.keys = (uint64_t*)malloc(e.cap * sizeof(uint64_t));
        e.vals = (uint32_t*)malloc(e.cap * sizeof(uint32_t));
        memset(e.keys, 0xff, e.cap * sizeof(uint64_t));
        uint32_t* g = (uint32_t*)malloc(nf * 4 * sizeof(uint32_t));
        size_t ng = 0;
        for (size_t i = 0; i < nf; i += 3) {
            uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            uint32_t ab = edge_mid(&e, &p, &np, &pcap, a, b);
            uint32_t bc = edge_mid(&e, &p, &np, &pcap, b, c);
            uint32_t ca = edge_mid(&e, &p, &np, &pcap, c, a);
            uint32_t tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            memcpy(g + ng, tri, sizeof(tri));
            ng += 12;
        }
        free(e.keys);
        free(e.vals);
        free(f);
        f = g;
        nf = ng;
    }
    m->nv = np;
    m->nt = (uint32_t)(nf / 3);
    m->pos = (float*)malloc((size_t)np * 3 * sizeof(float));
    m->normal = (float*)malloc((size_t)np * 3 * sizeof(float));
    m->uv = (float*)malloc((size_t)np * 2 * sizeof(float));
    const double pi = 3.14159265358979323846;
    for (uint32_t i = 0; i < np; ++i) {
        for (int c = 0; c < 3; ++c) {
            m->pos[3 * (size_t)i + c] = (float)p[i][c];
            m->normal[3 * (size_t)i + c] = (float)p[i][c];
        }
        m->uv[2 * (size_t)i] = (float)(0.5 + atan2(p[i][2], p[i][0]) / (2 * pi));
        double y = p[i][1] < -1.0 ? -1.0 : (p[i][1] > 1.0 ? 1.0 : p[i][1]);
        m->uv[2 * (size_t)i + 1] = (float)(acos(y) / pi);
    }
    m->idx = f;
    double* out = (double*)malloc((size_t)m->nt * 3 * sizeof(double));
    for (uint32_t tri = 0; tri < m->nt; ++tri) {
        double o[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) o[c] += p[m->idx[3 * tri + k]][c];
        memcpy(out + 3 * (size_t)tri, o, sizeof(o));
    }
    orient(m, out);
    free(out);
    free(p);
    compute_aabb(m);
    fill_vertex_stream(m);
    return m;
}

int orc_mesh_displace(orc_mesh* m, float amp, uint64_t seed) {
    if (!m) return -1;
    for (uint32_t i = 0; i < m->nv; ++i) {
        double x = m->pos[3 * (size_t)i], y = m->pos[3 * (size_t)i + 1], z = m->pos[3 * (size_t)i + 2];
        double l = sqrt(x * x + y * y + z * z);
        if (l == 0) continue;
        double d = amp * noise3(seed, x * 4 + 11.5, y * 4 + 7.25, z * 4 + 3.125);
        double s = (l + d) / l;
        m->pos[3 * (size_t)i] = (float)(x * s);
        m->pos[3 * (size_t)i + 1] = (float)(y * s);
        m->pos[3 * (size_t)i + 2] = (float)(z * s);
    }
    compute_aabb(m);
    fill_vertex_stream(m);
    clear_meshlets(m);
    return 0;
}

/* ----------------------------------------------------------------- torus */

orc_mesh* orc_mesh_torus(float R, float r, uint32_t seg_major, uint32_t seg_minor, float noise_amp, uint64_t seed,
                         int32_t quantize) {
    if (seg_major < 3 || seg_minor < 3 || seg_major > 4096 || seg_minor > 4096) return NULL;
    orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
    m->position_scale = 1.0f;
    const double pi = 3.14159265358979323846;
    const uint32_t nu = seg_major + 1, nvv = seg_minor + 1;
    double lat[200];
    {
        uint64_t s = seed;
        for (int i = 0; i < 200; ++i) lat[i] = rng_sym(&s);
    }
    const size_t nv = (size_t)nu * nvv;
    double* P = (double*)malloc(nv * 3 * sizeof(double));
    double* N = (double*)malloc(nv * 3 * sizeof(double));
    for (uint32_t j = 0; j < nvv; ++j)
        for (uint32_t i = 0; i < nu; ++i) {
            double s = (double)i / seg_major, t = (double)j / seg_minor;
            double u = 2 * pi * s, v = 2 * pi * t;
            double n[3] = {cos(v) * cos(u), sin(v), cos(v) * sin(u)};
            double d = r + noise_amp * noise2(lat, 20, 10, s, t);
            size_t k = ((size_t)j * nu + i) * 3;
            P[k] = R * cos(u) + d * n[0];
            P[k + 1] = d * n[1];
            P[k + 2] = R * sin(u) + d * n[2];
            for (int c = 0; c < 3; ++c) N[k + c] = n[c];
        }
    m->nv = (uint32_t)nv;
    m->pos = (float*)malloc(nv * 3 * sizeof(float));
    m->normal = (float*)malloc(nv * 3 * sizeof(float));
    m->uv = (float*)malloc(nv * 2 * sizeof(float));
    double maxabs = 0;
    for (size_t k = 0; k < nv * 3; ++k) maxabs = fabs(P[k]) > maxabs ? fabs(P[k]) : maxabs;
    if (quantize) {
        /* KHR_mesh_quantization: SHORT normalised positions, BYTE normals */
        double scale = ceil(maxabs * 64.0) / 64.0;
        m->position_scale = (float)scale;
        for (size_t k = 0; k < nv * 3; ++k) {
            long q = lrint(P[k] / scale * 32767.0);
            q = q < -32767L ? -32767L : (q > 32767L ? 32767L : q);
            m->pos[k] = fmaxf_((float)q / 32767.0f, -1.0f);
            long qn = lrint(N[k] * 127.0);
            m->normal[k] = fmaxf_((float)qn / 127.0f, -1.0f);
        }
    } else {
        for (size_t k = 0; k < nv * 3; ++k) {
            m->pos[k] = (float)P[k];
            m->normal[k] = (float)N[k];
        }
    }
    for (uint32_t j = 0; j < nvv; ++j)
        for (uint32_t i = 0; i < nu; ++i) {
            m->uv[2 * ((size_t)j * nu + i)] = (float)((double)i / seg_major);
            m->uv[2 * ((size_t)j * nu + i) + 1] = (float)((double)j / seg_minor);
        }
    /* quads in 7 x 7 blocks */
    m->nt = 2 * seg_major * seg_minor;
    m->idx = (uint32_t*)malloc((size_t)m->nt * 3 * sizeof(uint32_t));
    size_t w = 0;
    const uint32_t B = 7;
    for (uint32_t bj = 0; bj < seg_minor; bj += B)
        for (uint32_t bi = 0; bi < seg_major; bi += B)
            for (uint32_t j = bj; j < (bj + B < seg_minor ? bj + B : seg_minor); ++j)
                for (uint32_t i = bi; i < (bi + B < seg_major ? bi + B : seg_major); ++i) {
                    uint32_t a = j * nu + i, b = j * nu + i + 1, c = (j + 1) * nu + i + 1, d = (j + 1) * nu + i;
                    uint32_t q[6] = {a, b, c, a, c, d};
                    memcpy(m->idx + w, q, sizeof(q));
                    w += 6;
                }
    double* out = (double*)malloc((size_t)m->nt * 3 * sizeof(double));
    for (uint32_t tri = 0; tri < m->nt; ++tri) {
        double o[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) o[c] += N[(size_t)m->idx[3 * tri + k] * 3 + c];
        memcpy(out + 3 * (size_t)tri, o, sizeof(o));
    }
    orient(m, out);
    free(out);
    free(P);
    free(N);
    compute_aabb(m);
    fill_vertex_stream(m);
    return m;
}

/* ------------------------------------------------------------ meshletiser */

/* normal cone of a meshlet: cutoff rounded down, radius rounded up; cutoff
 * -1 (never culled) for a degenerate triangle or a cone wider than ~87 deg */
static orc_cone meshlet_cone(const orc_mesh* m, const uint32_t* tris, size_t ntris, const uint32_t* verts,
                             size_t nverts, const float* center, double* normals) {
    orc_cone cone;
    memset(&cone, 0, sizeof(cone));
    for (int c = 0; c < 3; ++c) cone.center[c] = center[c];
    double r2 = 0;
    for (size_t i = 0; i < nverts; ++i) {
        double d2 = 0;
        for (int c = 0; c < 3; ++c) {
            double e = (double)m->pos[3 * (size_t)verts[i] + c] - (double)center[c];
            d2 += e * e;
        }
        r2 = d2 > r2 ? d2 : r2;
    }
    double rr = sqrt(r2) * (1.0 + 1e-6) + 1e-7;
    cone.radius = nextafterf((float)rr, INFINITY);
    cone.cutoff = -1.0f;
    double sum[3] = {0, 0, 0};
    for (size_t i = 0; i < ntris; ++i) {
        uint32_t t = tris[i];
        const float* a = &m->pos[3 * (size_t)m->idx[3 * t]];
        const float* b = &m->pos[3 * (size_t)m->idx[3 * t + 1]];
        const float* c = &m->pos[3 * (size_t)m->idx[3 * t + 2]];
        double e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = (double)b[k] - a[k];
            e2[k] = (double)c[k] - a[k];
        }
        double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (!(len > 1e-30)) return cone;
        for (int k = 0; k < 3; ++k) {
            n[k] /= len;
            normals[3 * i + k] = n[k];
            sum[k] += n[k];
        }
    }
    double sl = sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
    if (!(sl > 1e-12)) return cone;
    double axis[3] = {sum[0] / sl, sum[1] / sl, sum[2] / sl};
    double cmin = 1.0;
    for (size_t i = 0; i < ntris; ++i) {
        double d = normals[3 * i] * axis[0] + normals[3 * i + 1] * axis[1] + normals[3 * i + 2] * axis[2];
        cmin = d < cmin ? d : cmin;
    }
    if (!(cmin > 0.05)) return cone;
    for (int k = 0; k < 3; ++k) cone.axis[k] = (float)axis[k];
    double cmin_f = 1.0;
    double fa[3] = {cone.axis[0], cone.axis[1], cone.axis[2]};
    double fal = sqrt(fa[0] * fa[0] + fa[1] * fa[1] + fa[2] * fa[2]);
    for (size_t i = 0; i < ntris; ++i) {
        double d = (normals[3 * i] * fa[0] + normals[3 * i + 1] * fa[1] + normals[3 * i + 2] * fa[2]) / fal;
        cmin_f = d < cmin_f ? d : cmin_f;
    }
    cmin_f -= 1e-6;
    if (!(cmin_f > 0.05)) return cone;
    cone.cutoff = nextafterf((float)cmin_f, -INFINITY);
    return cone;
}

/* Greedy adjacency-driven meshletiser: grows one meshlet at a time under the
 * vertex and triangle limits, always adding the candidate triangle that
 * brings the fewest new vertices (first found on ties), and starts a new
 * meshlet at the lowest unused triangle when none fits. */
int orc_mesh_build_meshlets(orc_mesh* m, uint32_t max_v, uint32_t max_t) {
    if (!m || max_v < 3 || max_v > 255 || max_t < 1 || max_t > 255) return -1;
    clear_meshlets(m);
    const size_t nv = m->nv, nt = m->nt;
    uint32_t* off = (uint32_t*)calloc(nv + 1, sizeof(uint32_t));
    uint32_t* adj = (uint32_t*)malloc((nt > 0 ? nt * 3 : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < nt * 3; ++i) off[m->idx[i] + 1]++;
    for (size_t v = 0; v < nv; ++v) off[v + 1] += off[v];
    {
        uint32_t* fill = (uint32_t*)malloc((nv ? nv : 1) * sizeof(uint32_t));
        memcpy(fill, off, nv * sizeof(uint32_t));
        for (size_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) adj[fill[m->idx[3 * t + k]]++] = (uint32_t)t;
        free(fill);
    }
    uint8_t* used = (uint8_t*)calloc(nt ? nt : 1, 1);
    int32_t* local = (int32_t*)malloc((nv ? nv : 1) * sizeof(int32_t));
    for (size_t v = 0; v < nv; ++v) local[v] = -1;
    uint32_t* stamp = (uint32_t*)calloc(nt ? nt : 1, sizeof(uint32_t));
    uint32_t cur = 0;
    size_t seed = 0, remaining = nt;
    uint32_t* mverts = (uint32_t*)malloc(256 * sizeof(uint32_t));
    uint32_t* mtris = (uint32_t*)malloc(256 * sizeof(uint32_t));
    double* normals = (double*)malloc(256 * 3 * sizeof(double));
    size_t ccap = 1024, nc = 0;
    uint32_t* cand = (uint32_t*)malloc(ccap * sizeof(uint32_t));
    size_t mcap = nt / 32 + 16, vcap = nt + 64, pcap = nt * 3 + 64;
    m->meshlets = (orc_meshlet*)malloc(mcap * sizeof(orc_meshlet));
    m->cones = (orc_cone*)malloc(mcap * sizeof(orc_cone));
    m->vtx_idx = (uint32_t*)malloc(vcap * sizeof(uint32_t));
    m->prim_idx = (uint8_t*)malloc(pcap);
    while (remaining > 0) {
        while (used[seed]) ++seed;
        ++cur;
        size_t nmv = 0, nmt = 0;
        nc = 0;
#define ADD_TRI(tt)                                                              \
    do {                                                                         \
        uint32_t t_ = (tt);                                                      \
        used[t_] = 1;                                                            \
        --remaining;                                                             \
        mtris[nmt++] = t_;                                                       \
        for (int k_ = 0; k_ < 3; ++k_) {                                         \
            uint32_t v_ = m->idx[3 * t_ + k_];                                   \
            if (local[v_] < 0) {                                                 \
                local[v_] = (int32_t)nmv;                                        \
                mverts[nmv++] = v_;                                              \
                for (uint32_t e_ = off[v_]; e_ < off[v_ + 1]; ++e_) {            \
                    uint32_t u_ = adj[e_];                                       \
                    if (!used[u_] && stamp[u_] != cur) {                         \
                        stamp[u_] = cur;                                         \
                        if (nc == ccap) {                                        \
                            ccap *= 2;                                           \
                            cand = (uint32_t*)realloc(cand, ccap * sizeof(uint32_t)); \
                        }                                                        \
                        cand[nc++] = u_;                                         \
                    }                                                            \
                }                                                                \
            }                                                                    \
        }                                                                        \
    } while (0)
        ADD_TRI((uint32_t)seed);
        while (nmt < max_t) {
            int best = -1, best_new = 4;
            size_t w = 0;
            for (size_t i = 0; i < nc; ++i) {
                uint32_t u = cand[i];
                if (used[u]) continue;
                cand[w++] = u;
                int nn = 0;
                for (int k = 0; k < 3; ++k) nn += local[m->idx[3 * u + k]] < 0;
                if (nn < best_new) {
                    best_new = nn;
                    best = (int)u;
                }
            }
            nc = w;
            if (best < 0 || nmv + (size_t)best_new > max_v) break;
            ADD_TRI((uint32_t)best);
        }
#undef ADD_TRI
        if (m->meshlet_count == mcap) {
            mcap *= 2;
            m->meshlets = (orc_meshlet*)realloc(m->meshlets, mcap * sizeof(orc_meshlet));
            m->cones = (orc_cone*)realloc(m->cones, mcap * sizeof(orc_cone));
        }
        while (m->vtx_idx_count + nmv > vcap) {
            vcap *= 2;
            m->vtx_idx = (uint32_t*)realloc(m->vtx_idx, vcap * sizeof(uint32_t));
        }
        while (m->prim_idx_bytes + nmt * 3 + 4 > pcap) {
            pcap *= 2;
            m->prim_idx = (uint8_t*)realloc(m->prim_idx, pcap);
        }
        orc_meshlet ml;
        memset(&ml, 0, sizeof(ml));
        ml.vertex_offset = m->vtx_idx_count;
        ml.triangle_offset = m->prim_idx_bytes;
        ml.vertex_count = (uint8_t)nmv;
        ml.triangle_count = (uint8_t)nmt;
        memcpy(m->vtx_idx + m->vtx_idx_count, mverts, nmv * sizeof(uint32_t));
        m->vtx_idx_count += (uint32_t)nmv;
        for (size_t i = 0; i < nmt; ++i)
            for (int k = 0; k < 3; ++k) m->prim_idx[m->prim_idx_bytes++] = (uint8_t)local[m->idx[3 * mtris[i] + k]];
        while (m->prim_idx_bytes & 3u) m->prim_idx[m->prim_idx_bytes++] = 0;
        /* meshlet AABB from its vertices (assets.cpp:348-372) */
        float mn[3], mx[3];
        for (int c = 0; c < 3; ++c) mn[c] = mx[c] = m->pos[3 * (size_t)mverts[0] + c];
        for (size_t i = 1; i < nmv; ++i)
            for (int c = 0; c < 3; ++c) {
                float x = m->pos[3 * (size_t)mverts[i] + c];
                mn[c] = fminf_(mn[c], x);
                mx[c] = fmaxf_(mx[c], x);
            }
        for (int c = 0; c < 3; ++c) {
            float ctr = (mn[c] + mx[c]) * 0.5f;
            ml.aabb_center[c] = ctr;
            ml.aabb_extents[c] = mx[c] - ctr;
        }
        m->meshlets[m->meshlet_count] = ml;
        m->cones[m->meshlet_count] = meshlet_cone(m, mtris, nmt, mverts, nmv, ml.aabb_center, normals);
        m->meshlet_count++;
        for (size_t i = 0; i < nmv; ++i) local[mverts[i]] = -1;
    }
    free(off);
    free(adj);
    free(used);
    free(local);
    free(stamp);
    free(mverts);
    free(mtris);
    free(normals);
    free(cand);
    return 0;
}

int orc_mesh_get_info(const orc_mesh* m, orc_mesh_info* out) {
    if (!m || !out) return -1;
    memset(out, 0, sizeof(*out));
    out->vertex_count = m->nv;
    out->triangle_count = m->nt;
    out->meshlet_count = m->meshlet_count;
    out->vertex_index_count = m->vtx_idx_count;
    out->primitive_index_bytes = m->prim_idx_bytes;
    out->position_scale = m->position_scale;
    out->vertices = m->verts;
    out->positions = m->pos;
    out->uvs = m->uv;
    out->indices = m->idx;
    out->meshlets = m->meshlets;
    out->vertex_indices = m->vtx_idx;
    out->primitive_indices = m->prim_idx;
    out->cones = m->cones;
    for (int c = 0; c < 3; ++c) {
        out->aabb_extents[c] = m->aabb_ext[c];
        out->aabb_center[c] = m->aabb_ctr[c];
    }
    return 0;
}

/* ---------------------------------------------------------------- camera */

/* column-major 4x4 product, m[c*4 + r], float accumulation in k order */
static void mul4(const float* a, const float* b, float* r) {
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float s = 0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = s;
        }
}

/* plane k = row 3 +/- row {0,1,2} of VP, normalised by |xyz|, w negated
 * (camera.cpp:70-84) */
int orc_frustum_planes(const float* vp, float* out) {
    for (int k = 0; k < 6; ++k) {
        int row = k / 2;
        float sgn = (k & 1) ? -1.f : 1.f;
        float pl[4];
        for (int i = 0; i < 4; ++i) pl[i] = vp[i * 4 + 3] + sgn * vp[i * 4 + row];
        float len = sqrtf(pl[0] * pl[0] + pl[1] * pl[1] + pl[2] * pl[2]);
        if (!(len > 0)) return -1;
        for (int i = 0; i < 4; ++i) pl[i] /= len;
        pl[3] = -pl[3];
        for (int i = 0; i < 4; ++i) out[k * 4 + i] = pl[i];
    }
    return 0;
}

/* VP = reverseZ * perspectiveRH_ZO (Y flipped) * lookAtRH; current matrices
 * shift to the prev slots first (camera.cpp:38-48, 170-193) */
int orc_camera_update(orc_camera* cam, const float* eye, const float* target, const float* up, float fovy,
                      float aspect, float znear, float zfar) {
    if (!cam || !eye || !target || !up) return -1;
    if (!(fovy > 0 && fovy < 3.14159f) || !(aspect > 0) || !(znear > 0) || !(zfar > znear)) return -1;
    float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
    float fl = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0)) return -1;
    for (int i = 0; i < 3; ++i) f[i] /= fl;
    float s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    float sl = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (!(sl > 0)) return -1;
    for (int i = 0; i < 3; ++i) s[i] /= sl;
    float u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    float view[16] = {0};
    for (int i = 0; i < 3; ++i) {
        view[i * 4 + 0] = s[i];
        view[i * 4 + 1] = u[i];
        view[i * 4 + 2] = -f[i];
    }
    view[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    view[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    view[14] = (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2]);
    view[15] = 1.f;
    const float th = tanf(fovy / 2.f);
    float proj[16] = {0};
    proj[0] = 1.f / (aspect * th);
    proj[5] = -(1.f / th);
    proj[10] = zfar / (znear - zfar);
    proj[11] = -1.f;
    proj[14] = -(zfar * znear) / (zfar - znear);
    float rz[16] = {0};
    rz[0] = 1.f;
    rz[5] = 1.f;
    rz[10] = -1.f;
    rz[14] = 1.f;
    rz[15] = 1.f;
    float rp[16], vp[16];
    mul4(rz, proj, rp);
    mul4(rp, view, vp);
    memcpy(cam->prev_vp, cam->vp, 64);
    memcpy(cam->prev_occlusion_vp, cam->occlusion_vp, 64);
    memcpy(cam->vp, vp, 64);
    memcpy(cam->occlusion_vp, vp, 64);
    return orc_frustum_planes(vp, &cam->frustum[0][0]);
}
