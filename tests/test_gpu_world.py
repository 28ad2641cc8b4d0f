"""The device world update (vkgv_world_*, world.cpp:187-345): transforms
bit-identical to the oracle's recursive walk at many animation times, the
MeshletDraw list bit-identical at the full torus-grid size (2,057 nodes,
843,776 draws), hand trees with a node reached twice, meshless nodes and
empty primitives, a frame rendered from the device-built buffers, an animated
scene through one captured frame graph, and the argument checks."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, scene
from vk_gltf_viewer_gb300.renderer import ViewBuffers
from vk_gltf_viewer_gb300.world import DeviceWorld, HostWorld, grid_world, make_nodes

from gpu_util import Pair, oracle_flags, small_grid, u32, u64
from test_oracle_world import hand_world

pytestmark = pytest.mark.gpu

TIMES = [0.0, 0.37, 1.0, 1.3, 2.5, 3.999, 5.3, -0.5, 123.456]


def _transforms(renderer, dw: DeviceWorld, time: float) -> np.ndarray:
    out = torch.full((max(1, dw.transform_count) * 16,), float("nan"), dtype=torch.float32, device="cuda")
    dw.update_transforms(time, out)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(-1, 16)[: dw.transform_count]


def _draws(renderer, dw: DeviceWorld) -> np.ndarray:
    out = torch.full((max(1, dw.draw_count) * 3,), -1, dtype=torch.int32, device="cuda")
    dw.build_draws(out)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32).reshape(-1, 3)[: dw.draw_count]


def _same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_grid_world_matches_oracle(renderer):
    mesh = scene.torus(seed=7)
    host = grid_world(mesh.meshlet_count, mesh.position_scale)
    dw = DeviceWorld(renderer, host)
    try:
        assert dw.transform_count == 2048
        assert dw.draw_count == 2048 * mesh.meshlet_count == host.meshlet_draw_count
        d = _draws(renderer, dw)
        assert np.array_equal(d, ob.world_draws(host))
        for t in TIMES:
            got = _transforms(renderer, dw, t)
            exp = ob.world_transforms(host, t)
            bad = np.flatnonzero((got.view(np.uint32) != exp.view(np.uint32)).any(1))
            assert bad.size == 0, (t, bad[:5], got[bad[:1]], exp[bad[:1]])
        assert renderer.device_status() == (0, 0)
    finally:
        dw.close()


def test_hand_tree_matches_oracle(renderer):
    host = hand_world()
    dw = DeviceWorld(renderer, host)
    try:
        assert (dw.transform_count, dw.draw_count) == (5, host.meshlet_draw_count)
        assert np.array_equal(_draws(renderer, dw), ob.world_draws(host))
        for t in TIMES:
            assert _same_bits(_transforms(renderer, dw, t), ob.world_transforms(host, t)), t
    finally:
        dw.close()


def test_empty_and_meshless_worlds(renderer):
    nodes = make_nodes(3)
    nodes[0]["first_child"], nodes[0]["child_count"] = 0, 2
    for roots in ([], [0]):
        host = HostWorld(nodes=nodes, children=np.array([1, 2], np.uint32), roots=np.array(roots, np.uint32),
                         mesh_primitives=[[0]], primitive_meshlet_counts=np.array([5], np.uint32))
        dw = DeviceWorld(renderer, host)
        try:
            assert (dw.transform_count, dw.draw_count) == (0, 0)
            dw.update_transforms(0.5, torch.zeros(16, device="cuda"))
            dw.build_draws(torch.zeros(3, dtype=torch.int32, device="cuda"))
            torch.cuda.synchronize()
        finally:
            dw.close()


def test_frame_from_device_world(renderer):
    """The small torus grid rendered from buffers the world kernels wrote
    matches the oracle frame rendered from the oracle's walk."""
    base = small_grid()
    mesh = base.meshes[0]
    world = grid_world(mesh.meshlet_count, mesh.position_scale, grid=(4, 4, 2))
    time = 1.3
    host = scene.HostScene(meshes=base.meshes, prim_materials=base.prim_materials, materials=base.materials,
                           transforms=ob.world_transforms(world, time), node_meshes=[[0]] * 32,
                           textures=base.textures, draws=ob.world_draws(world))
    pair = Pair(host)
    dw = DeviceWorld(renderer, world)
    try:
        pair.dev.transforms.zero_()
        pair.dev.draws.zero_()
        dw.update_transforms(time, pair.dev.transforms)
        dw.build_draws(pair.dev.draws)
        centre = scene.grid_centre() * 0.25
        eye = centre + np.array([7.0, 4.0, 6.0])
        cam = scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, 1.6)
        flags = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.RESOLVE_FLAT | abi.WRITE_IDS
        v = ViewBuffers.allocate(320, 200, cam, host.draw_count)
        renderer.frame(pair.dev, [v], flags)
        torch.cuda.synchronize()
        e = ob.frame(pair.orc, cam, 320, 200, oracle_flags(flags))
        assert (u64(v.depth_id) != 0).sum() > 2000
        assert np.array_equal(u64(v.depth_id), e["depth_id"])
        assert np.array_equal(u32(v.visbuffer), e["ids"])
    finally:
        dw.close()


def test_world_argument_checks(renderer):
    lib = abi.load()

    def create(host):
        h = C.c_void_p()
        d = host.desc()
        return lib.vkgv_world_create(renderer.ctx, C.byref(d), C.byref(h)), h

    nodes = make_nodes(2)
    nodes[0]["first_child"], nodes[0]["child_count"] = 0, 1
    nodes[1]["first_child"], nodes[1]["child_count"] = 1, 1
    cyclic = HostWorld(nodes=nodes, children=np.array([1, 0], np.uint32), roots=np.array([0], np.uint32),
                       mesh_primitives=[[0]], primitive_meshlet_counts=np.array([1], np.uint32))
    assert create(cyclic)[0] == abi.LIMIT_EXCEEDED
    bad_child = HostWorld(nodes=nodes, children=np.array([1, 7], np.uint32), roots=np.array([0], np.uint32),
                          mesh_primitives=[[0]], primitive_meshlet_counts=np.array([1], np.uint32))
    assert create(bad_child)[0] == abi.INVALID_ARG
    host = hand_world()
    host.channels[1, 0] = 99  # sampler index out of range
    assert create(host)[0] == abi.INVALID_ARG
    host = hand_world()
    host.channels[1, 2] = abi.PATH_TRANSLATION  # a rotation sampler on a translation path
    assert create(host)[0] == abi.INVALID_ARG
    dw = DeviceWorld(renderer, hand_world())
    try:
        small = torch.zeros(3 * (dw.draw_count - 1), dtype=torch.int32, device="cuda")
        with pytest.raises(abi.VkgvError, match="capacity"):
            dw.build_draws(small)
        buf = torch.zeros(16 * dw.transform_count + 4, dtype=torch.float32, device="cuda")
        rc = lib.vkgv_world_update_transforms(renderer.ctx, dw.handle, C.c_float(0.0), buf.data_ptr() + 4,
                                              torch.cuda.current_stream().cuda_stream)
        assert rc == abi.INVALID_ARG
    finally:
        dw.close()


def test_animated_scene_through_a_captured_graph(renderer):
    """Per-frame animation in batched mode: the world kernels rewrite the
    transforms between launches of one captured two-view frame graph, and
    each launch matches the oracle frame at that animation time."""
    import dataclasses

    from vk_gltf_viewer_gb300.renderer import DeviceScene, ViewBuffers

    base = small_grid()
    mesh = base.meshes[0]
    world = grid_world(mesh.meshlet_count, mesh.position_scale, grid=(4, 4, 2))
    host = dataclasses.replace(base, transforms=ob.world_transforms(world, 0.0), draws=ob.world_draws(world))
    dev = DeviceScene(host, "cuda")
    dw = DeviceWorld(renderer, world)
    centre = scene.grid_centre() * 0.25
    cams, sizes = [], [(240, 160), (160, 200)]
    for off in ((7.0, 4.0, 6.0), (-6.0, 3.0, 7.5)):
        eye = centre + np.array(off)
        cams.append(scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, 1.5))
    views = [ViewBuffers.allocate(w, h, c, host.draw_count) for c, (w, h) in zip(cams, sizes)]
    flags = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.RESOLVE_FLAT | abi.WRITE_IDS
    try:
        dw.build_draws(dev.draws)
        dw.update_transforms(0.0, dev.transforms)
        g = renderer.capture(dev, views, flags)
        try:
            for t in (0.3, 1.7, 2.9):
                dw.update_transforms(t, dev.transforms)
                g.launch()
                torch.cuda.synchronize()
                osc = ob.OracleScene(dataclasses.replace(host, transforms=ob.world_transforms(world, t)))
                for v, cam in zip(views, cams):
                    e = ob.frame(osc, cam, v.width, v.height, oracle_flags(flags))
                    assert np.array_equal(u32(v.visbuffer), e["ids"]), t
            assert renderer.device_status() == (0, 0)
        finally:
            g.close()
    finally:
        dw.close()
