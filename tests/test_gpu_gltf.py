"""A glTF asset end to end: the small torus grid written as a .glb (node
tree, animations, a material with KHR_texture_transform), imported, its
transforms and draw list written by the world kernels at an animation time,
rendered on the device and compared with the oracle frame of the same
imported scene (transforms and draws from the oracle's walk)."""
import dataclasses

import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, gltf, scene
from vk_gltf_viewer_gb300.renderer import ViewBuffers
from vk_gltf_viewer_gb300.world import grid_world

from vk_gltf_viewer_gb300.gltf_export import write_world
from gpu_util import oracle_flags, rgba_close, small_grid, u32, u64

pytestmark = pytest.mark.gpu

def test_imported_asset_renders_like_the_oracle(renderer, tmp_path):
    base = small_grid()
    mesh = base.meshes[0]
    src_world = grid_world(mesh.meshlet_count, mesh.position_scale, grid=(4, 4, 2))
    material = {"pbrMetallicRoughness": {"baseColorTexture": {
        "index": 0, "extensions": {"KHR_texture_transform": {"scale": [4.0, 4.0]}}}}}
    path = write_world(tmp_path / "grid.glb", [mesh], src_world, material)
    host, world = gltf.load(path, texture_references=True)
    host.textures = base.textures
    assert len(host.meshes) == 1 and world.nodes.size == src_world.nodes.size
    assert host.meshes[0].meshlet_count == mesh.meshlet_count
    time = 1.3
    dev, dw = gltf.device_scene(renderer, host, world, animation_time=time)
    try:
        assert (dw.transform_count, dw.draw_count) == (32, 32 * mesh.meshlet_count)
        exp_t = ob.world_transforms(world, time)
        got_t = dev.transforms.cpu().numpy().view(np.float32).reshape(-1, 16)
        assert np.array_equal(got_t.view(np.uint32), exp_t.view(np.uint32))
        ohost = dataclasses.replace(host, transforms=exp_t, draws=ob.world_draws(world))
        osc = ob.OracleScene(ohost)
        centre = scene.grid_centre() * 0.25
        eye = centre + np.array([6.0, 5.0, 7.0])
        cam = scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, 1.6)
        flags = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.RESOLVE_TEXTURED | abi.WRITE_IDS
        v = ViewBuffers.allocate(320, 200, cam, host.draw_count)
        renderer.frame(dev, [v], flags)
        torch.cuda.synchronize()
        e = ob.frame(osc, cam, 320, 200, oracle_flags(flags))
        assert (u64(v.depth_id) != 0).sum() > 2000
        assert np.array_equal(u64(v.depth_id), e["depth_id"])
        assert np.array_equal(u32(v.visbuffer), e["ids"])
        ok, bad = rgba_close(u32(v.color), e["rgba"])
        assert ok, bad
        assert renderer.device_status() == (0, 0)
    finally:
        dw.close()
