"""Parity at the benchmark's full size: the 82M-triangle torus grid at
1920x1080 with two-pass occlusion culling and the textured resolve, in the
steady state the benchmark times (previous frame's pyramid), plus a batch of
uneven views as in the batched leg.  Visibility IDs, depth|id, survivor sets
and HiZ mips must be bit-exact; RGBA within 1/255."""
import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, scene

from gpu_util import Pair, oracle_flags, rgba_close, u32, u64, view

pytestmark = pytest.mark.gpu

FLAGS = (abi.CULL_FRUSTUM | abi.CULL_CONE | abi.CULL_OCCLUSION | abi.CULL_TWO_PASS | abi.BUILD_PYRAMID
         | abi.RESOLVE_TEXTURED | abi.WRITE_IDS)


@pytest.fixture(scope="module")
def full(renderer):
    return Pair(scene.scene_torus_grid())


def test_full_size_frame_bit_exact(renderer, full):
    w, h = 1920, 1080
    cam = scene.grid_camera(w, h)
    first = ob.frame(full.orc, cam, w, h, oracle_flags(FLAGS))
    exp = ob.frame(full.orc, cam, w, h, oracle_flags(FLAGS), prev_pyramid=first["pyramid"])
    v = view(full, cam, w, h, prev=first["pyramid"])
    renderer.frame(full.dev, [v], FLAGS)
    torch.cuda.synchronize()
    assert full.host.triangle_count == 81_920_000
    assert np.array_equal(np.sort(v.survivor_list()), np.sort(exp["survivors"]))
    assert np.array_equal(u64(v.depth_id), exp["depth_id"])
    assert np.array_equal(u32(v.visbuffer), exp["ids"])
    assert np.array_equal(v.pyramid.cpu().numpy()[: exp["pyramid"].size], exp["pyramid"])
    ok, bad = rgba_close(u32(v.color), exp["rgba"])
    assert ok, f"{bad} pixels off by more than 1/255"
    assert renderer.device_status() == (0, 0)


def test_full_size_batched_views_bit_exact(renderer, full):
    """Twenty of the 256 batched poses in one launch: the first four poses of
    each of the five resolutions (256^2, 512x384, 1024x576, 1280x720,
    1920x1080), steady state, against the oracle."""
    picked, per = [], {}
    for cam, w, h in scene.batch_views(256, seed=3):
        if per.get((w, h), 0) < 4:
            per[(w, h)] = per.get((w, h), 0) + 1
            picked.append((cam, w, h))
    assert sorted(per.values()) == [4] * 5
    views, exps = [], []
    for cam, w, h in picked:
        first = ob.frame(full.orc, cam, w, h, oracle_flags(FLAGS))
        exps.append(ob.frame(full.orc, cam, w, h, oracle_flags(FLAGS), prev_pyramid=first["pyramid"]))
        views.append(view(full, cam, w, h, prev=first["pyramid"]))
    renderer.frame(full.dev, views, FLAGS)
    torch.cuda.synchronize()
    for v, e in zip(views, exps):
        assert np.array_equal(u32(v.visbuffer), e["ids"]), (v.width, v.height)
        assert np.array_equal(np.sort(v.survivor_list()), np.sort(e["survivors"])), (v.width, v.height)
        assert np.array_equal(v.pyramid.cpu().numpy()[: e["pyramid"].size], e["pyramid"])
        ok, bad = rgba_close(u32(v.color), e["rgba"])
        assert ok, f"{bad} pixels off by more than 1/255"
    assert renderer.device_status() == (0, 0)


def test_full_size_fine_occlusion_bit_exact(renderer, full):
    """The C2 frame and four batched poses with the fine occlusion test: the
    oracle's survivors, and the same ids as without it."""
    flags = FLAGS | abi.CULL_OCCLUSION_FINE
    poses = [(scene.grid_camera(1920, 1080), 1920, 1080)] + scene.batch_views(4, seed=3)
    views, base_views, exps = [], [], []
    for cam, w, h in poses:
        first = ob.frame(full.orc, cam, w, h, oracle_flags(FLAGS))
        exps.append(ob.frame(full.orc, cam, w, h, oracle_flags(flags), prev_pyramid=first["pyramid"]))
        views.append(view(full, cam, w, h, prev=first["pyramid"]))
        base_views.append(view(full, cam, w, h, prev=first["pyramid"]))
    renderer.frame(full.dev, views, flags)
    renderer.frame(full.dev, base_views, FLAGS)
    torch.cuda.synchronize()
    for v, b, e in zip(views, base_views, exps):
        assert np.array_equal(np.sort(v.survivor_list()), np.sort(e["survivors"])), (v.width, v.height)
        assert np.array_equal(u32(v.visbuffer), e["ids"])
        assert np.array_equal(u32(v.visbuffer), u32(b.visbuffer))
        assert v.survivor_list().size < b.survivor_list().size


def test_all_256_batched_views_equal_single_view_frames(renderer, full):
    """Every one of the benchmark's 256 uneven poses, rendered together in one
    batched frame (steady state, each view reading its own previous pyramid,
    fine occlusion test on as in the benchmark), equals the same pose
    rendered alone through the single-view path: depth|id, visibility ids,
    colour, pyramid and survivor set bit for bit.  With the twenty poses
    checked against the oracle above, this carries the oracle's parity to
    the whole batch."""
    from vk_gltf_viewer_gb300.renderer import ViewBuffers

    flags = FLAGS | abi.CULL_OCCLUSION_FINE
    poses = scene.batch_views(256, seed=3)

    def make():
        out = []
        for cam, w, h in poses:
            vb = ViewBuffers.allocate(w, h, cam, full.host.draw_count, prev_pyramid="alias")
            vb.use_prev = False
            out.append(vb)
        return out

    batched, single = make(), make()
    renderer.frame(full.dev, batched, flags)
    for vb in batched:
        vb.use_prev = True
    renderer.frame(full.dev, batched, flags)
    for vb in single:
        renderer.frame(full.dev, [vb], flags)
        vb.use_prev = True
        renderer.frame(full.dev, [vb], flags)
    torch.cuda.synchronize()
    assert renderer.device_status() == (0, 0)
    for i, (a, b) in enumerate(zip(batched, single)):
        where = (i, a.width, a.height)
        assert torch.equal(a.depth_id, b.depth_id), where
        assert torch.equal(a.visbuffer, b.visbuffer), where
        assert torch.equal(a.color, b.color), where
        assert torch.equal(a.pyramid, b.pyramid), where
        na, nb = int(a.survivor_count.item()), int(b.survivor_count.item())
        assert na == nb, where
        assert torch.equal(torch.sort(a.survivors[:na])[0], torch.sort(b.survivors[:nb])[0]), where
