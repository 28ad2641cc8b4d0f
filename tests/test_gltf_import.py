"""The glTF 2.0 importer (vkgv_gltf_*, the fastgltf-based import of
assets.cpp:288-552 and World::addAsset): float and KHR_mesh_quantization
positions, u8/u16/u32 and generated indices, colours and UVs, strided and
sparse accessors, materials (index + 1, the default at 0,
KHR_texture_transform), node matrices decomposed into TRS, the first scene's
roots, animations of every interpolation and path; .glb, .gltf with a data
URI and with an external .bin; the errors the importer reports."""
import math

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, gltf, scene
from vk_gltf_viewer_gb300.world import quat_axis_angle

from vk_gltf_viewer_gb300.gltf_export import SHORT, Builder, quantize_i16

f32 = np.float32


def _trs_matrix(t, q, s) -> np.ndarray:
    x, y, z, w = (float(v) for v in q)
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(s, np.float64)[None, :]
    M[:3, 3] = t
    return M


def make_asset():
    """Returns (Builder, expectations)."""
    rng = np.random.default_rng(12)
    b = Builder()
    ico = scene.icosphere(2)
    ipos = ico.positions.astype(f32)
    rgba8 = rng.integers(0, 256, (ipos.shape[0], 4), dtype=np.uint8)
    uv = rng.random((ipos.shape[0], 2)).astype(f32)
    soup = rng.normal(size=(12, 3)).astype(f32)  # 4 triangles without an index accessor
    tor = scene.torus(R=1.0, r=0.35, seg_major=40, seg_minor=20, noise_amp=0.0)
    q, qs = quantize_i16(tor.positions.astype(np.float64))
    exp_tor = np.maximum(q.astype(f32) / f32(32767), f32(-1))
    mesh0 = {"primitives": [
        {"attributes": {"POSITION": b.accessor(ipos, minmax=True), "COLOR_0": b.accessor(rgba8, normalized=True),
                        "TEXCOORD_0": b.accessor(uv)},
         "indices": b.accessor(ico.indices.reshape(-1).astype(np.uint32)), "material": 0},
        {"attributes": {"POSITION": b.accessor(soup, minmax=True)}, "material": 1}]}
    mesh1 = {"primitives": [{"attributes": {"POSITION": b.accessor(q, normalized=True, minmax=True)},
                             "indices": b.accessor(tor.indices.reshape(-1).astype(np.uint16))}]}
    b.add("meshes", mesh0)
    b.add("meshes", mesh1)
    b.add("materials", {"pbrMetallicRoughness": {
        "baseColorFactor": [0.8, 0.5, 0.25, 1.0],
        "baseColorTexture": {"index": 0, "extensions": {"KHR_texture_transform": {
            "offset": [0.25, 0.5], "rotation": 0.3, "scale": [4.0, 2.0]}}}},
        "alphaCutoff": 0.3, "doubleSided": True, "name": "nöde ☃ \U0001F600"})
    b.add("materials", {})
    b.add("textures", {"source": 0})
    b.add("images", {"uri": "albedo.png"})
    t1, q1, s1 = np.array([1.0, -2.0, 0.5]), quat_axis_angle((1, 2, 3), 0.7), np.array([2.0, 0.5, 1.5])
    m1 = _trs_matrix(t1, q1, s1)
    b.add("nodes", {"children": [1, 2], "translation": [0.0, 1.0, 0.0]})
    b.add("nodes", {"mesh": 0, "matrix": [float(x) for x in m1.T.reshape(16)]})
    b.add("nodes", {"mesh": 1, "scale": [qs, qs, qs], "children": [3], "rotation": list(map(float, quat_axis_angle((0, 1, 0), 1.1)))})
    b.add("nodes", {"mesh": 0, "translation": [3.0, 0.0, 0.0]})
    b.add("nodes", {"mesh": 1})  # not in the scene
    b.gltf["scenes"] = [{"nodes": [0]}, {"nodes": [4]}]
    b.gltf["scene"] = 0
    b.gltf["extensionsUsed"] = ["KHR_mesh_quantization", "KHR_texture_transform"]
    b.gltf["extensionsRequired"] = ["KHR_mesh_quantization"]
    times = np.array([0.0, 1.0, 2.0], f32)
    tr = rng.normal(size=(3, 3)).astype(f32)
    rq = np.stack([quat_axis_angle((0, 0, 1), a) for a in (0.0, 0.5, 1.0)])
    rq16 = np.round(rq * 32767).astype(np.int16)
    cub = rng.normal(size=(9, 3)).astype(f32)
    wts = np.array([0.0, 1.0, 0.5], f32)
    a_t = b.accessor(times, minmax=True)
    b.add("animations", {"samplers": [{"input": a_t, "output": b.accessor(tr)},
                                      {"input": a_t, "output": b.accessor(rq16, normalized=True),
                                       "interpolation": "STEP"}],
                         "channels": [{"sampler": 0, "target": {"node": 2, "path": "translation"}},
                                      {"sampler": 1, "target": {"node": 3, "path": "rotation"}}]})
    b.add("animations", {"samplers": [{"input": a_t, "output": b.accessor(cub), "interpolation": "CUBICSPLINE"},
                                      {"input": a_t, "output": b.accessor(wts)}],
                         "channels": [{"sampler": 0, "target": {"node": 1, "path": "scale"}},
                                      {"sampler": 1, "target": {"node": 1, "path": "weights"}}]})
    exp = dict(ico=ico, ipos=ipos, rgba8=rgba8, uv=uv, soup=soup, tor=tor, exp_tor=exp_tor, qs=qs, t1=t1, q1=q1,
               s1=s1, tr=tr, rq=np.maximum(rq16.astype(f32) / f32(32767), f32(-1)), cub=cub, wts=wts, times=times)
    return b, exp


def _tri_set(mesh) -> set:
    """Triangles rebuilt from the meshlets, each rotated to start at its
    smallest index (orientation kept)."""
    out = set()
    for ml in mesh.meshlets:
        vo, to = int(ml["vertex_offset"]), int(ml["triangle_offset"])
        for t in range(int(ml["triangle_count"])):
            tri = [int(mesh.vertex_indices[vo + int(mesh.primitive_indices[to + 3 * t + k])]) for k in range(3)]
            r = tri.index(min(tri))
            out.add(tuple(tri[r:] + tri[:r]))
    return out


def _idx_set(idx) -> set:
    out = set()
    for tri in np.asarray(idx).reshape(-1, 3).tolist():
        r = tri.index(min(tri))
        out.add(tuple(tri[r:] + tri[:r]))
    return out


def check_import(host, world, exp, texture_references=False):
    assert len(host.meshes) == 3 and host.prim_materials == [1, 2, 0]
    p0, p1, p2 = host.meshes
    assert np.array_equal(p0.positions, exp["ipos"])
    assert np.array_equal(p0.indices.reshape(-1), exp["ico"].indices.reshape(-1))
    assert np.array_equal(p0.vertices["color"], exp["rgba8"])
    assert np.array_equal(p0.uvs, exp["uv"])
    assert np.array_equal(p1.positions, exp["soup"])
    assert np.array_equal(p1.indices.reshape(-1), np.arange(12))
    assert np.array_equal(p2.positions, exp["exp_tor"])
    assert np.array_equal(p2.indices.reshape(-1), exp["tor"].indices.reshape(-1))
    for m in host.meshes:
        assert _tri_set(m) == _idx_set(m.indices)
        assert int(m.meshlets["vertex_count"].max()) <= 64 and int(m.meshlets["triangle_count"].max()) <= 124
    mats = host.materials
    assert mats.shape == (3,)
    assert np.allclose(mats[0]["albedo_factor"], 1.0) and mats[0]["albedo_index"] == abi.INVALID_HANDLE
    assert np.allclose(mats[1]["albedo_factor"], [0.8, 0.5, 0.25, 1.0])
    assert np.isclose(mats[1]["alpha_cutoff"], 0.3) and mats[1]["double_sided"] == 1
    if texture_references:
        assert mats[1]["albedo_index"] == 0
        assert np.allclose(mats[1]["uv_offset"], [0.25, 0.5]) and np.allclose(mats[1]["uv_scale"], [4.0, 2.0])
        assert np.isclose(mats[1]["uv_rotation"], 0.3)
    else:
        assert mats[1]["albedo_index"] == abi.INVALID_HANDLE and np.allclose(mats[1]["uv_scale"], 1.0)
    assert mats[2]["double_sided"] == 0 and np.isclose(mats[2]["alpha_cutoff"], 0.5)
    n = world.nodes
    assert n.size == 5 and list(world.roots) == [0]
    assert np.allclose(n[1]["translation"], exp["t1"], atol=1e-6)
    assert np.allclose(n[1]["scale"], exp["s1"], atol=1e-6)
    assert np.allclose(np.abs(n[1]["rotation"] @ exp["q1"]), 1.0, atol=1e-6)  # q or -q
    assert np.allclose(n[0]["translation"], [0, 1, 0]) and np.allclose(n[0]["rotation"], [0, 0, 0, 1])
    assert np.allclose(n[2]["scale"], exp["qs"])
    assert n[4]["mesh_index"] == 1 and n[0]["mesh_index"] == abi.INVALID_HANDLE
    kids = lambda i: list(world.children[int(n[i]["first_child"]):int(n[i]["first_child"] + n[i]["child_count"])])
    assert kids(0) == [1, 2] and kids(2) == [3] and kids(3) == []
    assert world.mesh_primitives == [[0, 1], [2]]
    assert list(world.primitive_meshlet_counts) == [m.meshlet_count for m in host.meshes]
    s = world.samplers
    assert len(s) == 4
    assert np.array_equal(s[0].input, exp["times"]) and np.array_equal(s[0].output, exp["tr"])
    assert s[1].interpolation == abi.INTERP_STEP and np.array_equal(s[1].output, exp["rq"])
    assert s[2].interpolation == abi.INTERP_CUBICSPLINE and np.array_equal(s[2].output, exp["cub"])
    assert s[3].components == 1 and np.array_equal(s[3].output[:, 0], exp["wts"])
    ch = world.channels.tolist()
    assert ch == [[0, 2, abi.PATH_TRANSLATION, 0], [1, 3, abi.PATH_ROTATION, 0], [2, 1, abi.PATH_SCALE, 0],
                  [3, 1, abi.PATH_WEIGHTS, 0]]
    # depth-first slots: node 1 (mesh 0), node 2 (mesh 1), node 3 (mesh 0); node 4 is outside the scene
    assert world.visits() == [1, 2, 3]
    d = world.draw_list()
    assert np.array_equal(d, ob.world_draws(world))
    assert np.array_equal(host.draws, d) and host.transforms.shape == (3, 16)
    # the imported tree animates like any other (the oracle's walk runs on it)
    assert ob.world_transforms(world, 0.7).shape == (3, 16)


def test_glb(built, tmp_path):
    b, exp = make_asset()
    host, world = gltf.load(b.write_glb(tmp_path / "asset.glb"))
    check_import(host, world, exp)


def test_texture_references(built, tmp_path):
    b, exp = make_asset()
    host, world = gltf.load(b.write_glb(tmp_path / "asset.glb"), texture_references=True)
    check_import(host, world, exp, texture_references=True)


def test_gltf_data_uri_and_external_bin(built, tmp_path):
    b, exp = make_asset()
    host, world = gltf.load(b.write_gltf(tmp_path / "embedded.gltf"))
    check_import(host, world, exp)
    b, exp = make_asset()
    host, world = gltf.load(b.write_gltf(tmp_path / "external.gltf", external="geometry data.bin"))
    check_import(host, world, exp)


def test_strided_and_sparse_accessors(built, tmp_path):
    b = Builder()
    pos = np.random.default_rng(1).normal(size=(9, 3)).astype(f32)
    over = np.array([[9.0, 9.0, 9.0], [-9.0, 0.0, 1.0]], f32)
    acc = b.accessor(pos, stride=20, sparse=(np.array([2, 7], np.uint32), over))
    b.add("meshes", {"primitives": [{"attributes": {"POSITION": acc}}]})
    b.add("nodes", {"mesh": 0})
    b.gltf["scenes"] = [{"nodes": [0]}]
    host, world = gltf.load(b.write_glb(tmp_path / "sparse.glb"))
    want = pos.copy()
    want[[2, 7]] = over
    assert np.array_equal(host.meshes[0].positions, want)
    assert host.prim_materials == [0] and host.materials.shape == (1,)


def _error(tmp_path, mutate, match):
    b, _ = make_asset()
    mutate(b)
    with pytest.raises(abi.VkgvError, match=match):
        gltf.load(b.write_glb(tmp_path / "bad.glb"))


def test_import_errors(built, tmp_path):
    _error(tmp_path, lambda b: b.gltf["meshes"][0]["primitives"][0]["attributes"].pop("POSITION"), "POSITION")
    _error(tmp_path, lambda b: b.gltf["meshes"][1]["primitives"][0].__setitem__("mode", 0), "TRIANGLES")
    _error(tmp_path, lambda b: b.gltf["extensionsRequired"].append("KHR_draco_mesh_compression"),
           "KHR_draco_mesh_compression")
    _error(tmp_path, lambda b: b.gltf["asset"].__setitem__("version", "1.0"), "glTF 2.0")
    _error(tmp_path, lambda b: b.gltf["nodes"][0]["children"].append(17), "child")
    _error(tmp_path, lambda b: b.gltf["accessors"][0].__setitem__("count", 10 ** 6), "exceeds")

    def bad_index(b):
        b.gltf["accessors"][b.gltf["meshes"][0]["primitives"][0]["indices"]]["componentType"] = SHORT
    _error(tmp_path, bad_index, "index accessors")
    good = make_asset()[0].write_glb(tmp_path / "ok.glb").read_bytes()
    (tmp_path / "cut.glb").write_bytes(good[:len(good) // 2])
    with pytest.raises(abi.VkgvError, match="GLB"):
        gltf.load(tmp_path / "cut.glb")
    (tmp_path / "broken.gltf").write_text('{"asset": {"version": "2.0"}, "nodes": [1, ]}')
    with pytest.raises(abi.VkgvError, match="JSON.*byte"):
        gltf.load(tmp_path / "broken.gltf")
    with pytest.raises(abi.VkgvError, match="cannot open"):
        gltf.load(tmp_path / "missing.glb")


def test_decompose_mirrored_matrix(built, tmp_path):
    """A mirroring node matrix decomposes into a negative x scale and the
    matching rotation (the product is the matrix again)."""
    b = Builder()
    b.add("meshes", {"primitives": [{"attributes": {"POSITION": b.accessor(np.eye(3, dtype=f32))}}]})
    t, q, s = np.array([0.5, 0.0, -1.0]), quat_axis_angle((0.3, 1, 0), 2.0), np.array([-1.5, 2.0, 0.25])
    M = _trs_matrix(t, q, s)
    b.add("nodes", {"mesh": 0, "matrix": [float(x) for x in M.T.reshape(16)]})
    b.gltf["scenes"] = [{"nodes": [0]}]
    _, world = gltf.load(b.write_glb(tmp_path / "m.glb"))
    nd = world.nodes[0]
    assert nd["scale"][0] < 0
    back = _trs_matrix(nd["translation"], nd["rotation"], nd["scale"])
    assert np.allclose(back, M, atol=2e-6)
    assert math.isclose(float(np.linalg.norm(nd["rotation"])), 1.0, abs_tol=1e-6)
