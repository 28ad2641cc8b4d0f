"""Pins the CPU oracle against the hand-derived known-answer fixtures in
tests/golden/ (made by tests/golden/make_kats.py with exact rational
arithmetic, independently of the oracle)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import binding as ob

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return json.loads((GOLDEN / name).read_text())


@pytest.mark.parametrize("case", load("kat_raster.json"), ids=lambda c: c["name"])
def test_raster_kat(built, case):
    w, h = case["w"], case["h"]
    depth = np.zeros(w * h, np.uint64)
    for t in case["tris"]:
        ob.raster_triangle(t[0], t[1], t[2], 5, w, h, depth)
    got = sorted([int(i % w), int(i // w)] for i in np.nonzero(depth)[0])
    assert got == case["expect"]
    lo = (depth[depth != 0] & 0xFFFFFFFF).astype(np.int64)
    assert np.all(lo == 6)  # id + 1


def test_split_square_covers_each_centre_once(built):
    cases = {c["name"]: c for c in load("kat_raster.json")}
    a, b = cases["split_square_lower"], cases["split_square_upper"]
    sa = {tuple(p) for p in a["expect"]}
    sb = {tuple(p) for p in b["expect"]}
    assert not (sa & sb)
    assert len(sa | sb) == 64


def test_raster_depth_is_constant_plane(built):
    c = load("kat_raster.json")[0]
    depth = ob.raster_triangle(*c["tris"][0], 0, 8, 8)
    z = (depth[depth != 0] >> 32).astype(np.uint32).view(np.float32)
    assert np.all(z == np.float32(0.5))


@pytest.mark.parametrize("case", load("kat_hiz.json"), ids=lambda c: f"{c['w']}x{c['h']}")
def test_hiz_kat(built, case):
    w, h = case["w"], case["h"]
    d = np.array(case["depth"], np.float32).reshape(-1)
    depth_id = (d.view(np.uint32).astype(np.uint64) << np.uint64(32)) | np.uint64(1)
    pyr = ob.hiz(depth_id, w, h)
    flat = np.concatenate([np.array(m, np.float32).reshape(-1) for m in case["mips"]]) if case["mips"] else \
        np.zeros(0, np.float32)
    assert pyr[: flat.size].tolist() == flat.tolist()


@pytest.mark.parametrize("case", load("kat_resolve.json"), ids=lambda c: str(c["albedo"]))
def test_resolve_srgb_kat(built, case):
    got = [ob.unorm8(ob.from_linear(c)) for c in case["albedo"][:3]] + [ob.unorm8(case["albedo"][3])]
    assert got == case["rgba8"]


def test_frustum_kat(built):
    k = load("kat_cull.json")
    for b in k["boxes"]:
        assert ob.frustum_visible(b["center"], b["extents"], k["planes"]) == b["frustum"], b["name"]


def test_min_sample_skips_texels_for_odd_sizes(built):
    # 5 texels sampled at the centre of texel 0 of a 2-texel level:
    # t = 0.25 * 5 - 0.5 = 0.75 -> texels 0 and 1 only.
    img = np.array([[0.9, 0.8, 0.1, 0.7, 0.6]], np.float32)
    assert ob.min_sample(img, 0.25, 0.5) == np.float32(0.8)
    assert ob.min_sample(img, 0.75, 0.5) == np.float32(0.6)
