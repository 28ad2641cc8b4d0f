"""The oracle's motion vectors (visbuffer.frag.glsl:38) on CPU: its binary16
conversion against numpy's round-to-nearest-even cast, zero motion for a
static camera, and the analytic screen shift of a fronto-parallel plane under
a camera translation."""
import math

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import scene


def _half_bits(vals: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return vals.astype(np.float32).astype(np.float16).view(np.uint16)


def test_half_rn_matches_numpy():
    rng = np.random.default_rng(5)
    mags = np.exp2(rng.uniform(-30.0, 17.0, 40000)).astype(np.float32)
    signs = np.where(rng.random(40000) < 0.5, -1.0, 1.0).astype(np.float32)
    # exact ties between binary16 neighbours (normal and subnormal) and the edges
    ties = np.array([1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 2.0 ** -24 * 1.5, 2.0 ** -24 * 2.5, 2.0 ** -25,
                     2.0 ** -25 * 1.0000001, 65504.0, 65519.99, 65520.0, 2.0 ** -14, 2.0 ** -14 * (1 - 2.0 ** -12),
                     0.0, -0.0, np.inf, -np.inf, 1e-45, 3.4e38], np.float32)
    vals = np.concatenate([mags * signs, ties, -ties])
    got = np.array([ob.half_rn(float(v)) for v in vals], np.uint16)
    assert np.array_equal(got, _half_bits(vals))
    assert ob.half_rn(float("nan")) & 0x7C00 == 0x7C00 and ob.half_rn(float("nan")) & 0x3FF


def _plane_scene(half: float = 4.0):
    """A double-sided square in the z = 0 plane, subdivided 8 x 8."""
    n = 9
    xs = np.linspace(-half, half, n, dtype=np.float32)
    px, py = np.meshgrid(xs, xs, indexing="xy")
    pos = np.stack([px.ravel(), py.ravel(), np.zeros(n * n, np.float32)], 1)
    idx = []
    for j in range(n - 1):
        for i in range(n - 1):
            a, b, c, d = j * n + i, j * n + i + 1, (j + 1) * n + i, (j + 1) * n + i + 1
            idx += [a, b, d, a, d, c]
    mesh = scene.mesh_from_arrays(pos, np.asarray(idx, np.uint32).reshape(-1, 3))
    mats = np.concatenate([scene.default_material(), scene.make_material(double_sided=True)])
    return scene.HostScene(meshes=[mesh], prim_materials=[1], materials=mats,
                           transforms=scene.to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])


def _motion(host, cam, w, h):
    osc = ob.OracleScene(host)
    depth = ob.frame(osc, cam, w, h, ob.CULL_FRUSTUM)["depth_id"]
    mv = ob.motion(osc, cam, w, h, depth).view(np.float16).astype(np.float32).reshape(h, w, 2)
    return depth.reshape(h, w) != 0, mv


def test_static_camera_has_zero_motion(built):
    host = _plane_scene()
    cam = scene.camera((0.3, -0.2, 5.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 4 / 3)
    covered, mv = _motion(host, cam, 64, 48)
    assert covered.sum() > 500
    assert not mv.any()


@pytest.mark.parametrize("shift", [(0.2, 0.0), (0.0, 0.15), (-0.1, 0.05)])
def test_translation_shifts_plane_uniformly(built, shift):
    """A camera translated by (dx, dy) parallel to a plane at distance d
    moves every point of it by NDC (P00 dx / d, -P11 dy / d): the projection's
    y axis points down (camera.cpp:177); motion = half of prev - current."""
    w, h, fovy, d = 80, 60, 60.0, 5.0
    dx, dy = shift
    prev = scene.camera((0.0, 0.0, d), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), fovy, w / h)
    cam = scene.camera((dx, dy, d), (dx, dy, 0.0), (0.0, 1.0, 0.0), fovy, w / h, prev=prev)
    covered, mv = _motion(_plane_scene(), cam, w, h)
    assert covered.sum() > 0.5 * w * h
    p11 = 1.0 / math.tan(math.radians(fovy) / 2)
    p00 = p11 / (w / h)
    exp = np.array([0.5 * p00 * dx / d, -0.5 * p11 * dy / d], np.float32)
    err = np.abs(mv[covered] - exp).max()
    assert err < 2e-4, err
    assert not mv[~covered].any()
