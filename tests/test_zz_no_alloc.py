"""vkgv_cull_static: the cull entry point for callers that cannot allocate
device memory (a frame loop under global-mode stream capture, or a plugin
whose host owns every allocation).  It keeps its scratch in a fixed device
array inside the library instead of a context.

Checked here through the C ABI against the existing context-based vkgv_cull
on the same inputs, over two calls in a row (the second call must not see
the first call's counters).  Survivor sets are integer results, so they must
match exactly.  This file is collected last so that a run stopping at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _survivors(v):
    n = int(v.survivor_count.item())
    return np.sort(v.survivors[:n].cpu().numpy().view(np.uint32))


def test_cull_static_matches_context_cull(built):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import binding as ob
    from vk_gltf_viewer_gb300 import abi, scene
    from vk_gltf_viewer_gb300.renderer import DeviceScene, Renderer, ViewBuffers

    lib = abi.load()
    host = scene.scene_torus_grid(texture_size=0, grid=(4, 4, 2))
    dev = DeviceScene(host, "cuda")
    w, h = 640, 360
    cam0 = scene.grid_camera(w, h)
    prev = ob.frame(ob.OracleScene(host), cam0, w, h, ob.CULL_FRUSTUM | ob.BUILD_PYRAMID)["pyramid"]
    centre = tuple(scene.grid_centre() * 0.25)
    cams = [scene.camera((0.9, 4.0, 4.5), centre, (0, 1, 0), 75.0, w / h, prev=cam0),
            scene.camera((-4.0, 2.0, -3.0), centre, (0, 1, 0), 75.0, w / h, prev=cam0)]
    flags = abi.CULL_FRUSTUM | abi.CULL_OCCLUSION | abi.CULL_TWO_PASS
    r = Renderer(0)
    try:
        for cam in cams:  # two calls in a row
            ref = ViewBuffers.allocate(w, h, cam, host.draw_count, prev_pyramid=True)
            got = ViewBuffers.allocate(w, h, cam, host.draw_count, prev_pyramid=True)
            for v in (ref, got):
                v.prev_pyramid.copy_(torch.from_numpy(prev).cuda())
            r.clear(dev, ref)
            r.cull(dev, ref, flags, 1)
            stream = torch.cuda.current_stream().cuda_stream
            sv = got.struct(host.draw_count)
            assert lib.vkgv_cull_static(C.byref(dev.scene), C.byref(sv), flags, 1, stream) == abi.OK
            torch.cuda.synchronize()
            a, b = _survivors(ref), _survivors(got)
            assert a.size > 0
            assert np.array_equal(a, b)
        # sizes beyond the fixed scratch are refused with a clear status
        big = abi.Scene.from_buffer_copy(dev.scene)
        big.meshlet_draw_count = 262145
        sv = got.struct(262145)
        sv.survivor_capacity = 262145
        assert lib.vkgv_cull_static(C.byref(big), C.byref(sv), flags, 1, 0) == abi.LIMIT_EXCEEDED
    finally:
        r.close()
