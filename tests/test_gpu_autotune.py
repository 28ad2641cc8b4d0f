"""Every launch shape the autotuner may pick (bin size {8, 16, 32} x
meshlets per CTA {1, 2, 4}) renders bit-identical visibility to the oracle,
and the tuner's sweep and cache behave."""
import json

import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, autotune, scene
from vk_gltf_viewer_gb300.renderer import Renderer

from gpu_util import Pair, oracle_flags, small_grid, u32, u64, view

pytestmark = pytest.mark.gpu

FLAGS = (abi.CULL_FRUSTUM | abi.CULL_CONE | abi.CULL_OCCLUSION | abi.CULL_TWO_PASS | abi.BUILD_PYRAMID
         | abi.RESOLVE_FLAT | abi.WRITE_IDS)


@pytest.fixture(scope="module")
def grid(renderer):
    return Pair(small_grid())


def _views(grid):
    sizes = [(640, 360), (256, 256), (97, 61)]
    centre = scene.grid_centre() * 0.25
    rng = np.random.default_rng(31)
    out = []
    for w, h in sizes:
        d = rng.normal(size=3)
        eye = centre + 8.0 * d / np.linalg.norm(d)
        cam = scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 75.0, w / h)
        out.append((cam, w, h))
    return out


@pytest.mark.parametrize("bin_size", [8, 16, 32])
@pytest.mark.parametrize("split", [1, 2, 4])
def test_every_candidate_matches_oracle(grid, bin_size, split):
    r = Renderer(0, bin_size=bin_size, meshlets_per_cta=split)
    try:
        cams = _views(grid)
        views = [view(grid, cam, w, h) for cam, w, h in cams]
        # two frames: the second reads the first frame's pyramid (two-pass HiZ)
        first = [ob.frame(grid.orc, cam, w, h, oracle_flags(FLAGS)) for cam, w, h in cams]
        for v in views:
            v.use_prev = False
        r.frame(grid.dev, views, FLAGS)
        torch.cuda.synchronize()
        for v, e in zip(views, first):
            assert np.array_equal(u32(v.visbuffer), e["ids"])
            assert np.array_equal(u64(v.depth_id), e["depth_id"])
        prevs = [v.pyramid.cpu().numpy().copy() for v in views]
        views2 = [view(grid, cam, w, h, prev=p) for (cam, w, h), p in zip(cams, prevs)]
        r.frame(grid.dev, views2, FLAGS)
        torch.cuda.synchronize()
        for v, (cam, w, h), p in zip(views2, cams, prevs):
            e = ob.frame(grid.orc, cam, w, h, oracle_flags(FLAGS), prev_pyramid=p)
            assert np.array_equal(u32(v.visbuffer), e["ids"])
            assert np.array_equal(np.sort(v.survivor_list()), np.sort(e["survivors"]))
        assert r.device_status() == (0, 0)
    finally:
        r.close()


def test_tune_sweeps_nine_candidates_and_caches(renderer, grid, tmp_path):
    cams = _views(grid)
    views = [view(grid, cam, w, h) for cam, w, h in cams]
    renderer.frame(grid.dev, views, FLAGS & ~(abi.CULL_OCCLUSION | abi.CULL_TWO_PASS))
    torch.cuda.synchronize()
    path = tmp_path / "tune.json"
    rec = autotune.tune(renderer, grid.dev, views, FLAGS & ~(abi.CULL_OCCLUSION | abi.CULL_TWO_PASS),
                        launches=2, path=path)
    assert not rec["cached"]
    shapes = {(e["bin_size"], e["meshlets_per_cta"]) for e in rec["table"]}
    assert shapes == {(b, m) for b in (8, 16, 32) for m in (1, 2, 4)}
    assert all(e["ms_per_launch"] > 0 for e in rec["table"])
    best = min(rec["table"], key=lambda e: e["ms_per_launch"])
    assert (rec["bin_size"], rec["meshlets_per_cta"]) == (best["bin_size"], best["meshlets_per_cta"])
    again = autotune.tune(renderer, grid.dev, views, FLAGS & ~(abi.CULL_OCCLUSION | abi.CULL_TWO_PASS),
                          launches=2, path=path)
    assert again["cached"] and again["bin_size"] == rec["bin_size"]
    assert rec["key"] in json.loads(path.read_text())
    tuned, _ = autotune.tuned_renderer(renderer, grid.dev, views, FLAGS & ~(abi.CULL_OCCLUSION | abi.CULL_TWO_PASS),
                                       path=path)
    try:
        assert (tuned.bin_size, tuned.meshlets_per_cta) == (rec["bin_size"], rec["meshlets_per_cta"])
    finally:
        tuned.close()
