"""The view-sharded adjoint as the benchmark runs it under N ranks, with two
CPU (gloo) ranks that share this one GPU: each rank computes the library's
gradients over its pixel-balanced shard of the views (sharding.shard_views),
copies them to host memory and joins one sum all-reduce
(sharding.allreduce_gradients).  No kernel of one rank waits on the other:
the only exchange is the host-side collective.  The summed gradients must
equal the library's single-process gradients over all views up to fp32
summation order, and the shards must cover every view once."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

SIZES = [(64, 48), (40, 40), (96, 64), (32, 32), (80, 80), (48, 36), (128, 72)]


def _problem():
    from vk_gltf_viewer_gb300 import diff, scene

    rng = np.random.default_rng(31)
    mesh = scene.icosphere(3)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    tex = rng.uniform(0, 1, size=(32, 32, 3)).astype(np.float32)
    sc = diff.DiffScene.create(mesh, colors, tex)
    cams, targets = [], []
    for w, h in SIZES:
        v = rng.normal(size=3)
        eye = 3.0 * v / np.linalg.norm(v)
        cams.append(scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, w / h))
        targets.append(rng.uniform(0, 1, size=w * h * 3).astype(np.float32))
    return sc, cams, targets


def _library_grads(renderer, sc, cams, targets, which):
    from vk_gltf_viewer_gb300 import diff

    views = [diff.DiffViewBuffers.allocate(SIZES[i][0], SIZES[i][1], cams[i]) for i in which]
    gp, gc, gt = torch.zeros_like(sc.positions), torch.zeros_like(sc.colors), torch.zeros_like(sc.texture)
    loss = torch.zeros(1, device="cuda")
    scale = 1.0 / (3 * sum(w * h for w, h in SIZES))
    if which:
        diff.backward(renderer, sc, views, gp, gc, gt, targets=[torch.from_numpy(targets[i]).cuda() for i in which],
                      scale=scale, loss=loss)
    torch.cuda.synchronize()
    return [t.cpu() for t in (gp, gc, gt, loss)]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    from vk_gltf_viewer_gb300.renderer import Renderer
    from vk_gltf_viewer_gb300.sharding import allreduce_gradients, shard_views

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = Renderer(0)
    try:
        sc, cams, targets = _problem()
        mine = shard_views([w * h for w, h in SIZES], world, rank)
        grads = _library_grads(r, sc, cams, targets, mine)
        allreduce_gradients(grads)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), *[g.numpy() for g in grads],
                 mine=np.asarray(mine, np.int64))
    finally:
        r.close()
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_adjoint_allreduce_equals_single_process(renderer, tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    sc, cams, targets = _problem()
    full = [g.numpy() for g in _library_grads(renderer, sc, cams, targets, list(range(len(SIZES))))]
    owned = []
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        owned += list(z["mine"])
        for k, ref in enumerate(full):
            got = z[f"arr_{k}"]
            # fp32 atomics in a different order on each side of the sum
            assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref) + 1e-12, k
    assert sorted(owned) == list(range(len(SIZES)))
    assert all(len(np.load(tmp_path / f"rank{r}.npz")["mine"]) > 0 for r in range(world))
