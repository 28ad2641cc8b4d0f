"""The oracle's scene producers (oracle/scene.c, oracle/scene.py) against the
product's (csrc/scene.cpp, scene.py): every buffer of the C1 icosphere and the
C2 torus grid, the camera buffers of the grid camera and of the 256 batched
poses, byte for byte.  The benchmark's reference arm builds its inputs with
the oracle's producers, so that it never loads the product library; this
test is what makes its inputs the same workload."""
import numpy as np
import pytest

from oracle import scene as osn
from vk_gltf_viewer_gb300 import scene

MESH_FIELDS = ["vertices", "positions", "uvs", "indices", "meshlets", "vertex_indices", "primitive_indices",
               "aabb_extents", "aabb_center", "cones"]


def _same_mesh(a, b):
    for f in MESH_FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape, f
        assert x.tobytes() == y.tobytes(), f
    assert a.position_scale == b.position_scale


@pytest.mark.parametrize("kind", ["torus_grid", "icosphere"])
def test_scene_buffers_identical(built, kind):
    if kind == "torus_grid":
        a, b = scene.scene_torus_grid(texture_size=256), osn.scene_torus_grid(texture_size=256)
    else:
        a, b = scene.scene_icosphere(6), osn.scene_icosphere(6)
    assert len(a.meshes) == len(b.meshes)
    for ma, mb in zip(a.meshes, b.meshes):
        _same_mesh(ma, mb)
    for f in ["transforms", "materials", "draws"]:
        assert getattr(a, f).tobytes() == getattr(b, f).tobytes(), f
    assert a.prim_materials == b.prim_materials
    assert [t.data.tobytes() for t in a.textures] == [t.data.tobytes() for t in b.textures]


@pytest.mark.parametrize("args", [dict(level=5), dict(level=4, displace=0.02, seed=9)])
def test_icosphere_variants_identical(built, args):
    _same_mesh(scene.icosphere(**args), osn.icosphere(**args))


def test_torus_unquantised_identical(built):
    _same_mesh(scene.torus(seg_major=40, seg_minor=20, quantize=False, seed=3),
               osn.torus(seg_major=40, seg_minor=20, quantize=False, seed=3))


def test_camera_buffers_identical(built):
    assert bytes(scene.grid_camera(1920, 1080)) == bytes(osn.grid_camera(1920, 1080))
    assert bytes(scene.camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 1280 / 720)) == \
        bytes(osn.icosphere_camera(1280, 720))
    for (c1, w1, h1), (c2, w2, h2) in zip(scene.batch_views(256), osn.batch_views(256)):
        assert (w1, h1) == (w2, h2)
        assert bytes(c1) == bytes(c2)
    assert np.array_equal(scene.grid_centre(), osn.grid_centre())
