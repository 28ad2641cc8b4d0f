// The reference's own shared GLSL headers, compiled in their C++ mode
// (shaders/common.h.glsl:6-28) against the stand-ins in ref_stub/, behind a
// C ABI for the tests: struct sizes and member offsets
// (shaders/mesh_common.h.glsl:20-126, shaders/visbuffer/visbuffer.h.glsl:37-56),
// packVisBuffer / unpackVisBuffer (visbuffer.h.glsl:58-65) and
// fromLinear / toLinear (shaders/srgb.h.glsl:9-41).  TEST INFRASTRUCTURE ONLY:
// built from the reference sources into oracle/_ref/ when they are present,
// never linked by the product.
#include <cstddef>
#include <cstdint>

#include <mesh_common.h.glsl>
#include <srgb.h.glsl>
#include <visbuffer/visbuffer.h.glsl>

namespace {
struct Entry {
    const char* name;
    std::uint32_t value;
};

#define SZ(T) {#T, (std::uint32_t)sizeof(glsl::T)}
#define OFF(T, m) {#T "." #m, (std::uint32_t)offsetof(glsl::T, m)}

const Entry kLayout[] = {
    SZ(Camera), OFF(Camera, prevViewProjection), OFF(Camera, prevOcclusionViewProjection),
    OFF(Camera, viewProjection), OFF(Camera, occlusionViewProjection), OFF(Camera, frustum),
    SZ(TaskPayload), OFF(TaskPayload, baseID), OFF(TaskPayload, deltaIDs),
    SZ(Meshlet), OFF(Meshlet, vertexOffset), OFF(Meshlet, triangleOffset), OFF(Meshlet, vertexCount),
    OFF(Meshlet, triangleCount), OFF(Meshlet, aabbExtents), OFF(Meshlet, aabbCenter),
    SZ(Vertex), OFF(Vertex, position), OFF(Vertex, color), OFF(Vertex, normal), OFF(Vertex, uv),
    SZ(MeshletDraw), OFF(MeshletDraw, primitiveIndex), OFF(MeshletDraw, meshletIndex),
    OFF(MeshletDraw, transformIndex),
    SZ(Primitive), OFF(Primitive, vertexIndexBuffer), OFF(Primitive, primitiveIndexBuffer),
    OFF(Primitive, vertexBuffer), OFF(Primitive, meshletBuffer), OFF(Primitive, aabbExtents),
    OFF(Primitive, aabbCenter), OFF(Primitive, meshletCount), OFF(Primitive, materialIndex),
    SZ(Material), OFF(Material, albedoFactor), OFF(Material, albedoIndex), OFF(Material, uvOffset),
    OFF(Material, uvScale), OFF(Material, uvRotation), OFF(Material, alphaCutoff), OFF(Material, doubleSided),
    SZ(VisbufferPushConstants), OFF(VisbufferPushConstants, drawBuffer),
    OFF(VisbufferPushConstants, meshletDrawCount), OFF(VisbufferPushConstants, transformBuffer),
    OFF(VisbufferPushConstants, primitiveBuffer), OFF(VisbufferPushConstants, cameraBuffer),
    OFF(VisbufferPushConstants, materialBuffer), OFF(VisbufferPushConstants, depthPyramid),
    SZ(VisbufferResolvePushConstants), OFF(VisbufferResolvePushConstants, visbufferHandle),
    OFF(VisbufferResolvePushConstants, outputImageHandle), OFF(VisbufferResolvePushConstants, drawBuffer),
    OFF(VisbufferResolvePushConstants, primitiveBuffer), OFF(VisbufferResolvePushConstants, materialBuffer),
    {"maxVertices", glsl::maxVertices}, {"maxPrimitives", glsl::maxPrimitives},
    {"maxMeshlets", glsl::maxMeshlets}, {"triangleBits", glsl::triangleBits},
    {"drawIndexBits", glsl::drawIndexBits}, {"visbufferClearValue", glsl::visbufferClearValue},
    {"invalidHandle", glsl::invalidHandle},
};
}  // namespace

extern "C" {

std::uint32_t ref_layout_count(void) { return sizeof(kLayout) / sizeof(kLayout[0]); }

const char* ref_layout_name(std::uint32_t i) { return i < ref_layout_count() ? kLayout[i].name : nullptr; }

std::uint32_t ref_layout_value(std::uint32_t i) { return i < ref_layout_count() ? kLayout[i].value : 0u; }

std::uint32_t ref_pack_visbuffer(std::uint32_t draw, std::uint32_t prim) { return glsl::packVisBuffer(draw, prim); }

void ref_unpack_visbuffer(std::uint32_t v, std::uint32_t* draw, std::uint32_t* prim) {
    glsl::uint d = 0, p = 0;
    glsl::unpackVisBuffer(v, d, p);
    *draw = d;
    *prim = p;
}

float ref_from_linear(float c) { return glsl::fromLinear(c); }

float ref_to_linear(float c) { return glsl::toLinear(c); }

void ref_from_linear4(const float* in, float* out) {
    glsl::vec4 r = glsl::fromLinear(glsl::vec4(in[0], in[1], in[2], in[3]));
    out[0] = r.x, out[1] = r.y, out[2] = r.z, out[3] = r.w;
}

void ref_to_linear4(const float* in, float* out) {
    glsl::vec4 r = glsl::toLinear(glsl::vec4(in[0], in[1], in[2], in[3]));
    out[0] = r.x, out[1] = r.y, out[2] = r.z, out[3] = r.w;
}
}
