"""Frames and adjoint passes of more views than the kernels' per-launch view
tables hold: the meshlet raster takes at most 1,024 views per launch (the
launcher splits larger batches), the chunked resolve and the persistent
adjoint shade at most 4,096 (larger calls take their per-view grid forms).
4,100 small views of uneven sizes cross both limits; every view must match
the oracle (ids and survivors bit-exact, RGBA within 1/255; adjoint images
and gradients against float64)."""
import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, diff, scene

from gpu_util import Pair, oracle_flags, rgba_close, u32, view

pytestmark = pytest.mark.gpu

NVIEWS = 4100


def _cameras(n, seed, sizes):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = rng.normal(size=3)
        eye = 3.0 * v / np.linalg.norm(v)
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        out.append((scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, w / h), w, h))
    return out


def test_frame_of_4100_views(renderer):
    host = scene.scene_icosphere(3)
    pair = Pair(host)
    flags = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.RESOLVE_FLAT | abi.WRITE_IDS | abi.BUILD_PYRAMID
    cams = _cameras(NVIEWS, 21, [(8, 8), (16, 8), (12, 20), (24, 24)])
    views = [view(pair, c, w, h) for c, w, h in cams]
    renderer.frame(pair.dev, views, flags)
    torch.cuda.synchronize()
    assert renderer.device_status() == (0, 0)
    drawn = 0
    for v, (c, w, h) in zip(views, cams):
        e = ob.frame(pair.orc, c, w, h, oracle_flags(flags))
        ids = u32(v.visbuffer)
        assert np.array_equal(ids, e["ids"]), (w, h)
        assert np.array_equal(np.sort(v.survivor_list()), np.sort(e["survivors"]))
        ok, bad = rgba_close(u32(v.color), e["rgba"])
        assert ok, bad
        drawn += int((ids != abi.VISBUFFER_CLEAR).sum())
    assert drawn > NVIEWS * 16


def test_adjoint_of_4100_views(renderer):
    rng = np.random.default_rng(23)
    mesh = scene.icosphere(3)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    texture = rng.uniform(0, 1, size=(32, 32, 3)).astype(np.float32)
    sc = diff.DiffScene.create(mesh, colors, texture)
    cams = _cameras(NVIEWS, 25, [(8, 8), (16, 12)])
    views = [diff.DiffViewBuffers.allocate(w, h, c) for c, w, h in cams]
    out = [torch.zeros(w * h * 3, device="cuda") for _, w, h in cams]
    diff.forward(renderer, sc, views, out)
    torch.cuda.synchronize()
    targets = [rng.uniform(0, 1, size=w * h * 3).astype(np.float32) for _, w, h in cams]
    scale = 1.0 / (3 * sum(w * h for _, w, h in cams))
    gp, gc, gt = torch.zeros_like(sc.positions), torch.zeros_like(sc.colors), torch.zeros_like(sc.texture)
    loss = torch.zeros(1, device="cuda")
    diff.backward(renderer, sc, views, gp, gc, gt, targets=[torch.from_numpy(t).cuda() for t in targets],
                  scale=scale, loss=loss)
    torch.cuda.synchronize()
    ref_loss, ref = 0.0, None
    for (c, w, h), v, o, t in zip(cams, views, out, targets):
        vp = np.frombuffer(bytes(c), np.float32)[32:48].copy()
        ids = v.ids()
        lv, rgb, g = ob.diff_f64(mesh, mesh.positions, colors, mesh.uvs, texture, vp, w, h, ids, target=t,
                                 scale=scale, want_rgb=True, want_grads=True)
        assert np.abs(o.cpu().numpy() - rgb).max() < 5e-4
        ref_loss += lv
        ref = g if ref is None else tuple(a + b for a, b in zip(ref, g))
    assert abs(float(loss.item()) - ref_loss) <= 1e-4 * abs(ref_loss)
    for name, g, r in (("positions", gp, ref[0]), ("colors", gc, ref[1]), ("texels", gt, ref[2])):
        g = g.cpu().numpy().reshape(-1)
        assert np.linalg.norm(g - r) / np.linalg.norm(r) < 1e-3, name
