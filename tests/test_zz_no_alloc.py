"""vkgv_cull_static: the cull entry point for callers that cannot allocate
device memory (a frame loop under global-mode stream capture, or a plugin
whose host owns every allocation).  It keeps its scratch in a fixed device
array inside the library instead of a context.

Checked here through the C ABI against the existing context-based vkgv_cull
on the same inputs, over two calls in a row (the second call must not see
the first call's counters), for pass 1 and for pass 2, which re-tests the
pass-1 occlusion rejects that the preceding pass-1 call left in the shared
array.  Pass 2 is also checked against the oracle.  Survivor sets are integer
results, so they must match exactly.  The status reader must report a draw
with an out-of-range meshlet index and then read clear.  This file is
collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _survivors(v):
    n = int(v.survivor_count.item())
    return v.survivors[:n].cpu().numpy().view(np.uint32).copy()


def _status(lib, stream):
    code, detail = C.c_uint32(7), C.c_uint32(7)
    assert lib.vkgv_cull_static_status(stream, C.byref(code), C.byref(detail)) == 0
    return int(code.value), int(detail.value)


def test_cull_static_matches_context_cull(built):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import binding as ob
    from vk_gltf_viewer_gb300 import abi, scene
    from vk_gltf_viewer_gb300.renderer import DeviceScene, Renderer, ViewBuffers

    lib = abi.load()
    host = scene.scene_torus_grid(texture_size=0, grid=(4, 4, 2))
    osc = ob.OracleScene(host)
    dev = DeviceScene(host, "cuda")
    w, h = 640, 360
    cam0 = scene.grid_camera(w, h)
    prev = ob.frame(osc, cam0, w, h, ob.CULL_FRUSTUM | ob.BUILD_PYRAMID)["pyramid"]
    centre = tuple(scene.grid_centre() * 0.25)
    cams = [scene.camera((0.9, 4.0, 4.5), centre, (0, 1, 0), 75.0, w / h, prev=cam0),
            scene.camera((-4.0, 2.0, -3.0), centre, (0, 1, 0), 75.0, w / h, prev=cam0)]
    flags = abi.CULL_FRUSTUM | abi.CULL_OCCLUSION | abi.CULL_TWO_PASS
    stream = torch.cuda.current_stream().cuda_stream
    r = Renderer(0)
    try:
        _status(lib, stream)  # start from clear status words
        for cam in cams:  # two calls in a row
            ref = ViewBuffers.allocate(w, h, cam, host.draw_count, prev_pyramid=True)
            got = ViewBuffers.allocate(w, h, cam, host.draw_count, prev_pyramid=True)
            for v in (ref, got):
                v.prev_pyramid.copy_(torch.from_numpy(prev).cuda())
            r.clear(dev, ref)
            r.cull(dev, ref, flags, 1)
            sv = got.struct(host.draw_count)
            assert lib.vkgv_cull_static(C.byref(dev.scene), C.byref(sv), flags, 1, stream) == abi.OK
            torch.cuda.synchronize()
            a, b = _survivors(ref), _survivors(got)
            assert a.size > 0
            assert np.array_equal(np.sort(a), np.sort(b))
            exp1, rej1 = ob.cull(osc, cam, w, h, ob.CULL_FRUSTUM | ob.CULL_OCCLUSION | ob.CULL_TWO_PASS, 1,
                                 pyramid=prev)
            assert np.array_equal(np.sort(b), np.sort(exp1))
            assert rej1.size > 0
            # pass 2 against this camera's own pyramid (the frame's rebuilt one)
            pyr = ob.frame(osc, cam, w, h, ob.CULL_FRUSTUM | ob.BUILD_PYRAMID)["pyramid"]
            for v in (ref, got):
                v.pyramid.copy_(torch.from_numpy(pyr).cuda())
            r.cull(dev, ref, flags, 2)
            sv = got.struct(host.draw_count)
            assert lib.vkgv_cull_static(C.byref(dev.scene), C.byref(sv), flags, 2, stream) == abi.OK
            torch.cuda.synchronize()
            a2, b2 = _survivors(ref), _survivors(got)
            assert b2.size == int(got.survivor_count.item())
            # pass-1 survivors stay first; pass 2 appends the re-tested rejects
            assert np.array_equal(b2[: b.size], b)
            assert np.array_equal(np.sort(a2), np.sort(b2))
            exp2, _ = ob.cull(osc, cam, w, h, ob.CULL_FRUSTUM | ob.CULL_OCCLUSION | ob.CULL_TWO_PASS, 2,
                              pyramid=pyr, candidates=rej1)
            assert np.array_equal(np.sort(b2[b.size:]), np.sort(exp2))
            assert _status(lib, stream) == (0, 0)
        # a device-side fault is reported by the status reader, then cleared
        bad = host.draws.copy()
        bad_draw = 5
        bad.reshape(-1, 3)[bad_draw, 1] = 1 << 20  # meshlet index far past the primitive's count
        bad_t = torch.from_numpy(bad.view(np.int32).ravel().copy()).cuda()
        bscene = abi.Scene.from_buffer_copy(dev.scene)
        bscene.draw_buffer = bad_t.data_ptr()
        sv = got.struct(host.draw_count)
        assert lib.vkgv_cull_static(C.byref(bscene), C.byref(sv), abi.CULL_FRUSTUM, 1, stream) == abi.OK
        assert _status(lib, stream) == (1, bad_draw)
        assert _status(lib, stream) == (0, 0)
        # sizes beyond the fixed scratch are refused with a clear status
        big = abi.Scene.from_buffer_copy(dev.scene)
        big.meshlet_draw_count = 262145
        sv = got.struct(262145)
        sv.survivor_capacity = 262145
        assert lib.vkgv_cull_static(C.byref(big), C.byref(sv), flags, 1, 0) == abi.LIMIT_EXCEEDED
    finally:
        r.close()
