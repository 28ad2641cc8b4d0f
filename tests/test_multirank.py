"""Multi-rank logic on CPU ranks (gloo, world size 2): view sharding and the
adjoint's gradient sum all-reduce.  Each rank computes the float64
reference gradient of the views it owns; after the all-reduce every rank
holds the gradient of all views."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from vk_gltf_viewer_gb300.sharding import allreduce_gradients, shard_views

SIZES = [(64, 48), (40, 40), (96, 64), (32, 32), (80, 80), (48, 36)]


def test_shard_views_partition_is_exact_and_balanced():
    px = [w * h for w, h in SIZES]
    for world in (1, 2, 3, 4, 8):
        parts = [shard_views(px, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(px)))
        loads = [sum(px[i] for i in p) for p in parts]
        # greedy LPT: no rank exceeds the mean by more than the largest view
        assert max(loads) <= sum(px) / world + max(px)
    assert shard_views([], 2, 1) == []
    with pytest.raises(ValueError):
        shard_views(px, 2, 2)
    with pytest.raises(ValueError):
        shard_views([-1], 1, 0)


def _problem():
    from oracle import binding as ob
    from vk_gltf_viewer_gb300 import scene

    rng = np.random.default_rng(21)
    mesh = scene.icosphere(2)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3))
    tex = rng.uniform(0, 1, size=(16, 16, 3))
    host = scene.HostScene(meshes=[mesh], prim_materials=[1],
                           materials=np.concatenate([scene.default_material(), scene.make_material()]),
                           transforms=scene.to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])
    osc = ob.OracleScene(host)
    views = []
    for w, h in SIZES:
        v = rng.normal(size=3)
        eye = 3.0 * v / np.linalg.norm(v)
        cam = scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, w / h)
        ids = ob.frame(osc, cam, w, h, 0)["ids"]
        target = rng.uniform(0, 1, size=w * h * 3).astype(np.float32)
        views.append((np.frombuffer(bytes(cam), np.float32)[32:48].copy(), w, h, ids, target))
    return mesh, colors, tex, views


def _grads(mesh, colors, tex, views, which):
    from oracle import binding as ob

    gp = np.zeros(mesh.positions.size)
    gc = np.zeros(colors.size)
    gt = np.zeros(tex.size)
    for i in which:
        vp, w, h, ids, target = views[i]
        _, _, (p, c, t) = ob.diff_f64(mesh, mesh.positions, colors, mesh.uvs, tex, vp, w, h, ids, target=target,
                                      scale=1e-3, want_grads=True)
        gp += p
        gc += c
        gt += t
    return gp, gc, gt


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mesh, colors, tex, views = _problem()
        mine = shard_views([w * h for _, w, h, _, _ in views], world, rank)
        grads = [torch.from_numpy(g) for g in _grads(mesh, colors, tex, views, mine)]
        allreduce_gradients(grads)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), *[g.numpy() for g in grads],
                 mine=np.asarray(mine, np.int64))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gradient_allreduce_equals_single_process(built, tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    mesh, colors, tex, views = _problem()
    full = _grads(mesh, colors, tex, views, range(len(views)))
    owned = []
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        owned += list(z["mine"])
        for k, ref in enumerate(full):
            # the sum over two ranks is the sum over all views, up to the
            # float64 reassociation of the per-view partial sums
            np.testing.assert_allclose(z[f"arr_{k}"], ref, rtol=1e-12, atol=1e-15)
    assert sorted(owned) == list(range(len(views)))


def test_allreduce_rejects_mixed_dtypes():
    with pytest.raises(ValueError):
        allreduce_gradients([torch.zeros(2, dtype=torch.float32), torch.zeros(2, dtype=torch.float64)])
