// Minimal stand-in for glm (absent: the reference's submodule is empty), with
// just what the reference's shared GLSL headers use in their C++ mode
// (shaders/common.h.glsl:6-28): the vector and matrix types with glm's
// default (packed, 4-byte aligned) layout, and the GLSL built-ins of
// shaders/srgb.h.glsl (pow, mix with a boolean selector, lessThan, the .rgb /
// .a views of a vec4).  Semantics follow the GLSL specification; glm
// implements the same.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cmath>
#include <cstdint>

namespace glm {

struct bvec3 {
    bool x, y, z;
};

struct vec2 {
    float x, y;
};

struct vec3 {
    float x, y, z;
    vec3() = default;
    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};

inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }

// The storage of a vec4's .rgb view: a plain aggregate (allowed in the
// anonymous union below) that converts to vec3 wherever one is expected.
struct vec3_view {
    float x, y, z;
    operator vec3() const { return vec3(x, y, z); }
};

struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        struct {
            vec3_view rgb;
            float a_;
        };
    };
    vec4() = default;
    constexpr vec4(float p, float q, float s, float t) : x(p), y(q), z(s), w(t) {}
    vec4(vec3 v, float t) : x(v.x), y(v.y), z(v.z), w(t) {}
};

struct mat4 {
    vec4 c[4];
};

struct u8vec3 {
    std::uint8_t x, y, z;
};
struct u8vec4 {
    std::uint8_t x, y, z, w;
};
struct u16vec2 {
    std::uint16_t x, y;
};

// GLSL mix(x, y, bool a): y where a is true, else x.
inline float mix(float x, float y, bool a) { return a ? y : x; }
inline vec3 mix(vec3 x, vec3 y, bvec3 a) { return vec3(a.x ? y.x : x.x, a.y ? y.y : x.y, a.z ? y.z : x.z); }
inline bvec3 lessThan(vec3 p, vec3 q) { return bvec3{p.x < q.x, p.y < q.y, p.z < q.z}; }
inline vec3 pow(vec3 p, vec3 q) { return vec3(std::pow(p.x, q.x), std::pow(p.y, q.y), std::pow(p.z, q.z)); }

static_assert(sizeof(vec3) == 12 && alignof(vec3) == 4, "glm vec3 layout");
static_assert(sizeof(vec4) == 16 && sizeof(mat4) == 64, "glm vec4/mat4 layout");
static_assert(sizeof(u16vec2) == 4 && sizeof(u8vec3) == 3, "glm small vector layout");

}  // namespace glm
