"""Motion vectors (visbuffer.frag.glsl:38, the visibility pass's R16G16_SFLOAT
attachment): the CUDA resolve's binary16 image is bit-identical to the
oracle's on the same depth|id image, through whole frames (node tables),
batched views, the resolve stage entry (no node tables) and a captured graph."""
import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, scene
from vk_gltf_viewer_gb300.renderer import ViewBuffers

from gpu_util import Pair, oracle_flags, small_grid, u32, u64

pytestmark = pytest.mark.gpu

BASE = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.WRITE_IDS | abi.WRITE_MOTION


@pytest.fixture(scope="module")
def grid(renderer):
    return Pair(small_grid())


def _moving_cameras(n: int, w: int, h: int, seed: int):
    """Cameras whose previous frame looked from a nearby eye at a nearby
    target (a translating and turning camera)."""
    rng = np.random.default_rng(seed)
    centre = scene.grid_centre() * 0.25
    out = []
    for _ in range(n):
        d = rng.normal(size=3)
        eye = centre + 8.0 * d / np.linalg.norm(d)
        prev_eye = eye + rng.normal(scale=0.4, size=3)
        prev_target = centre + rng.normal(scale=0.3, size=3)
        prev = scene.camera(tuple(prev_eye), tuple(prev_target), scene.safe_up(prev_eye, prev_target), 70.0, w / h)
        out.append(scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, w / h, prev=prev))
    return out


def _views(grid, cams, sizes):
    return [ViewBuffers.allocate(w, h, cam, grid.host.draw_count, motion=True) for cam, (w, h) in zip(cams, sizes)]


def _check(grid, v, cam):
    depth = u64(v.depth_id)
    exp = ob.motion(grid.orc, cam, v.width, v.height, depth)
    got = u32(v.motion)
    bad = np.flatnonzero(got != exp)
    assert bad.size == 0, (bad.size, bad[:5], got[bad[:5]], exp[bad[:5]])
    return depth, got


@pytest.mark.parametrize("shade", [0, abi.RESOLVE_FLAT, abi.RESOLVE_TEXTURED])
def test_frame_motion_matches_oracle(renderer, grid, shade):
    sizes = [(320, 200), (97, 61), (256, 256)]
    cams = _moving_cameras(len(sizes), 320, 200, seed=41)
    views = _views(grid, cams, sizes)
    flags = BASE | shade
    renderer.frame(grid.dev, views, flags)
    torch.cuda.synchronize()
    moving = 0
    for v, cam in zip(views, cams):
        e = ob.frame(grid.orc, cam, v.width, v.height, oracle_flags(flags))
        depth, got = _check(grid, v, cam)
        assert np.array_equal(depth, e["depth_id"])
        assert np.all(got[depth == 0] == 0)
        moving += int((got[depth != 0] != 0).sum())
    assert moving > 1000
    assert renderer.device_status() == (0, 0)


def test_static_camera_writes_zero(renderer, grid):
    centre = scene.grid_centre() * 0.25
    eye = centre + np.array([6.0, 3.0, 5.0])
    cam = scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, 1.5)
    v = ViewBuffers.allocate(300, 200, cam, grid.host.draw_count, motion=True)
    v.motion.fill_(-1)
    renderer.frame(grid.dev, [v], BASE)
    torch.cuda.synchronize()
    assert (u64(v.depth_id) != 0).sum() > 1000
    assert not u32(v.motion).any()


def test_stage_resolve_matches_frame(renderer, grid):
    """vkgv_resolve alone (prev_view_projection * M per pixel) writes the same
    image as the frame (node tables from the clear)."""
    cam = _moving_cameras(1, 240, 160, seed=7)[0]
    v = ViewBuffers.allocate(240, 160, cam, grid.host.draw_count, motion=True)
    renderer.frame(grid.dev, [v], BASE | abi.RESOLVE_TEXTURED)
    torch.cuda.synchronize()
    first = u32(v.motion).copy()
    v.motion.zero_()
    renderer.resolve(grid.dev, v, abi.WRITE_MOTION)
    torch.cuda.synchronize()
    assert np.array_equal(u32(v.motion), first)
    _check(grid, v, cam)


def test_captured_graph_matches(renderer, grid):
    cams = _moving_cameras(2, 200, 150, seed=9)
    views = _views(grid, cams, [(200, 150), (150, 200)])
    g = renderer.capture(grid.dev, views, BASE | abi.RESOLVE_FLAT)
    try:
        g.launch()
        torch.cuda.synchronize()
        for v, cam in zip(views, cams):
            _check(grid, v, cam)
    finally:
        g.close()


def test_motion_needs_an_image(renderer, grid):
    cam = _moving_cameras(1, 64, 64, seed=3)[0]
    v = ViewBuffers.allocate(64, 64, cam, grid.host.draw_count)
    with pytest.raises(abi.VkgvError, match="motion"):
        renderer.frame(grid.dev, [v], BASE)
