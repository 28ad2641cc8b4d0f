"""The reference's own code, compiled from its shared GLSL headers in their
C++ mode (shaders/common.h.glsl:6-28), against the library's ABI and the
oracle:

- struct sizes, member offsets and constants of shaders/mesh_common.h.glsl:
  20-126 and shaders/visbuffer/visbuffer.h.glsl:15-67 against include/vkgv.h
  (through its ctypes mirror, which test_abi.py pins to vkgv.h with a gcc
  probe);
- packVisBuffer / unpackVisBuffer (visbuffer.h.glsl:58-65) against the ids of
  an oracle frame (bit-identical to the kernels' ids in the GPU parity tests);
- fromLinear / toLinear (shaders/srgb.h.glsl:9-41) against the oracle's
  sRGB.  The vec4 forms, which the resolve applies to the albedo
  (visbuffer_resolve.comp.glsl:38), use float literals and match the oracle
  bit for bit.  The scalar forms write 1.055 and 12.92 unsuffixed, which GLSL
  evaluates in float and C++ (the headers' C++ mode) in double; the oracle
  follows the shader, so those agree to 2 ulp (fromLinear) and 1 ulp
  (toLinear), and exactly after the UNORM8 store on the fixture's sweep.

The checks run against tests/golden/ref_headers.json (written by
tests/golden/make_ref_vectors.py from the reference build) everywhere, and
also against the live reference build (oracle/_ref/) where the reference
sources are present."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "ref_headers.json").read_text())

# reference struct -> (vkgv.h ctypes mirror, {reference member: vkgv member})
STRUCTS = {
    "Camera": (abi.Camera, {"prevViewProjection": "prev_view_projection",
                            "prevOcclusionViewProjection": "prev_occlusion_view_projection",
                            "viewProjection": "view_projection",
                            "occlusionViewProjection": "occlusion_view_projection", "frustum": "frustum"}),
    "Meshlet": (abi.Meshlet, {"vertexOffset": "vertex_offset", "triangleOffset": "triangle_offset",
                              "vertexCount": "vertex_count", "triangleCount": "triangle_count",
                              "aabbExtents": "aabb_extents", "aabbCenter": "aabb_center"}),
    "Vertex": (abi.Vertex, {"position": "position", "color": "color", "normal": "normal", "uv": "uv"}),
    "MeshletDraw": (abi.MeshletDraw, {"primitiveIndex": "primitive_index", "meshletIndex": "meshlet_index",
                                      "transformIndex": "transform_index"}),
    "Primitive": (abi.Primitive, {"vertexIndexBuffer": "vertex_index_buffer",
                                  "primitiveIndexBuffer": "primitive_index_buffer", "vertexBuffer": "vertex_buffer",
                                  "meshletBuffer": "meshlet_buffer", "aabbExtents": "aabb_extents",
                                  "aabbCenter": "aabb_center", "meshletCount": "meshlet_count",
                                  "materialIndex": "material_index"}),
    "Material": (abi.Material, {"albedoFactor": "albedo_factor", "albedoIndex": "albedo_index",
                                "uvOffset": "uv_offset", "uvScale": "uv_scale", "uvRotation": "uv_rotation",
                                "alphaCutoff": "alpha_cutoff", "doubleSided": "double_sided"}),
}


def _layouts():
    out = [("golden", GOLDEN["layout"])]
    lib = ob.load_ref()
    if lib is not None:
        out.append(("live", ob.ref_layout(lib)))
    return out


def test_live_reference_build_matches_fixture(built):
    lib = ob.load_ref()
    if lib is None:
        pytest.skip("reference sources absent: the fixture alone is checked")
    assert ob.ref_layout(lib) == GOLDEN["layout"]
    xs = np.array(GOLDEN["srgb_inputs"], np.uint32).view(np.float32)
    fl = np.array([lib.ref_from_linear(float(x)) for x in xs], np.float32).view(np.uint32)
    tl = np.array([lib.ref_to_linear(float(x)) for x in xs], np.float32).view(np.uint32)
    assert fl.tolist() == GOLDEN["from_linear"]
    assert tl.tolist() == GOLDEN["to_linear"]
    assert len(GOLDEN["from_linear4"]) == xs.size and len(GOLDEN["to_linear4"]) == xs.size


@pytest.mark.parametrize("name", sorted(STRUCTS))
def test_struct_layout_matches_vkgv_h(name):
    cls, members = STRUCTS[name]
    for src, lay in _layouts():
        assert lay[name] == C.sizeof(cls), (src, name)
        for ref_m, our_m in members.items():
            assert lay[f"{name}.{ref_m}"] == getattr(cls, our_m).offset, (src, name, ref_m)


def test_constants_match_vkgv_h():
    for src, lay in _layouts():
        assert lay["maxVertices"] == abi.MAX_VERTICES, src
        assert lay["maxPrimitives"] == abi.MAX_PRIMITIVES, src
        assert lay["triangleBits"] == abi.TRIANGLE_BITS, src
        assert lay["drawIndexBits"] == 32 - abi.TRIANGLE_BITS, src
        assert lay["visbufferClearValue"] == 0xFFFFFFFF, src
        assert lay["invalidHandle"] == abi.INVALID_HANDLE, src
        # the task payload the warp compaction replaces: 4 + 102 bytes
        assert lay["TaskPayload.deltaIDs"] == 4 and lay["maxMeshlets"] == 102, src


def test_visbuffer_packing_matches_oracle_ids(built):
    for d, t, v, dd, tt in GOLDEN["pack"]:
        assert v == ((d << 7) | t) and (dd, tt) == (d, t)
    from oracle import scene as osn
    host = osn.scene_torus_grid(texture_size=0, grid=(4, 4, 2))
    osc = ob.OracleScene(host)
    w, h = 320, 180
    cam = osn.camera((-3.0, 4.0, -4.0), tuple(osn.grid_centre() * 0.25), (0.0, 1.0, 0.0), 60.0, w / h)
    f = ob.frame(osc, cam, w, h, ob.CULL_FRUSTUM | ob.RESOLVE_FLAT)
    ids = f["ids"]
    drawn = ids[ids != 0xFFFFFFFF]
    assert drawn.size > 1000
    # every id is a packVisBuffer of a survivor and a triangle of its meshlet
    draw, tri = drawn >> 7, drawn & 127
    assert np.isin(draw, f["survivors"]).all()
    counts = host.meshes[0].meshlets["triangle_count"][host.draws[draw, 1]]
    assert (tri < counts).all()
    lib = ob.load_ref()
    if lib is not None:
        sample = drawn[:: max(1, drawn.size // 2000)]
        for v in sample:
            dd, tt = C.c_uint32(), C.c_uint32()
            lib.ref_unpack_visbuffer(int(v), C.byref(dd), C.byref(tt))
            assert (dd.value, tt.value) == (int(v) >> 7, int(v) & 127)
            assert lib.ref_pack_visbuffer(dd.value, tt.value) == int(v)


def test_srgb_matches_oracle(built):
    lib = ob.load()
    xs = np.array(GOLDEN["srgb_inputs"], np.uint32).view(np.float32)
    ref_f = np.array(GOLDEN["from_linear"], np.uint32).view(np.float32)
    ref_t = np.array(GOLDEN["to_linear"], np.uint32).view(np.float32)
    orc_f = np.array([lib.orc_from_linear(float(x)) for x in xs], np.float32)
    orc_t = np.array([lib.orc_to_linear(float(x)) for x in xs], np.float32)

    def ulp(a, b):
        return np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))

    assert ulp(ref_f, orc_f).max() <= 2
    assert ulp(ref_t, orc_t).max() <= 1
    u = lambda arr: np.array([lib.orc_unorm8(float(x)) for x in arr])
    assert np.array_equal(u(ref_f), u(orc_f))
    assert np.array_equal(u(ref_t), u(orc_t))
    # the cut-offs select the same branch (linear segment below, power above)
    for x, f in zip(xs, orc_f):
        if x < np.float32(0.0031308):
            assert f == np.float32(x * np.float32(12.92))


def test_vec4_forms_match_oracle_exactly(built):
    lib = ob.load()
    xs = np.array(GOLDEN["srgb_inputs"], np.uint32).view(np.float32)
    orc_f = np.array([lib.orc_from_linear(float(x)) for x in xs], np.float32).view(np.uint32)
    orc_t = np.array([lib.orc_to_linear(float(x)) for x in xs], np.float32).view(np.uint32)
    assert orc_f.tolist() == GOLDEN["from_linear4"]
    assert orc_t.tolist() == GOLDEN["to_linear4"]
    ref = ob.load_ref()
    if ref is None:
        return
    rng = np.random.default_rng(3)
    for _ in range(200):
        v = rng.random(4).astype(np.float32)
        out = np.zeros(4, np.float32)
        ref.ref_from_linear4(v.ctypes.data, out.ctypes.data)
        assert out[:3].view(np.uint32).tolist() == [int(np.float32(lib.orc_from_linear(float(x))).view(np.uint32))
                                                     for x in v[:3]]
        assert out[3] == v[3]
        ref.ref_to_linear4(v.ctypes.data, out.ctypes.data)
        assert out[:3].view(np.uint32).tolist() == [int(np.float32(lib.orc_to_linear(float(x))).view(np.uint32))
                                                     for x in v[:3]]
        assert out[3] == v[3]
