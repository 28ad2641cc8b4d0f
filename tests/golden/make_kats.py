"""Generates the known-answer fixtures in this folder.

The answers are derived here from the rules themselves with exact rational
arithmetic (fractions.Fraction), independently of the C oracle and of the CUDA
kernels, on cases small enough to check by hand:

  kat_raster.json   coverage of hand-placed clip-space triangles under the
                    Vulkan rasterisation rules the path pins (pixel centres
                    at +0.5, 8 sub-pixel bits, top-left fill rule, near-plane
                    clipping of a crossing triangle);
  kat_hiz.json      HiZ reduce chains of small depth images, including odd
                    sizes (where the MIN-reduction footprint skips texels) and
                    a view whose top mip is never written (pinned to 0.0);
  kat_resolve.json  the flat resolve's sRGB-encoded RGBA8 of constant
                    base colours (shaders/srgb.h.glsl:9-15 with UNORM8 store);
  kat_cull.json     frustum and occlusion verdicts of boxes under an identity
                    view-projection, including a box face lying exactly on a
                    plane (shaders/culling.h.glsl:8-19, task.glsl:54-65).

Run:  python tests/golden/make_kats.py
"""
from __future__ import annotations

import json
import math
from fractions import Fraction as F
from pathlib import Path

HERE = Path(__file__).resolve().parent


# ----------------------------------------------------------------- raster

def snap(v: F) -> F:
    """Round to 1/256 with ties to even (8 sub-pixel bits)."""
    s = v * 256
    fl = math.floor(s)
    r = s - fl
    if r > F(1, 2) or (r == F(1, 2) and fl % 2 == 1):
        fl += 1
    return F(fl, 256)


def screen(v, w, h):
    x, y, z, wc = v
    return ((x / wc + 1) * F(w, 2), (y / wc + 1) * F(h, 2))


def coverage(verts, w, h):
    """Pixels whose centre the snapped polygon covers under the top-left rule
    (vertices given in screen space, any orientation)."""
    pts = [(snap(x), snap(y)) for x, y in verts]
    covered = set()
    for k in range(1, len(pts) - 1):
        tri = [pts[0], pts[k], pts[k + 1]]
        (x0, y0), (x1, y1), (x2, y2) = tri
        area = (x1 - x0) * (y2 - y0) - (y1 - y0) * (x2 - x0)
        if area == 0:
            continue
        if area < 0:
            tri = [tri[0], tri[2], tri[1]]
        for py in range(h):
            for px in range(w):
                sx, sy = F(2 * px + 1, 2), F(2 * py + 1, 2)
                ok = True
                for i in range(3):
                    (ax, ay), (bx, by) = tri[i], tri[(i + 1) % 3]
                    e = (bx - ax) * (sy - ay) - (by - ay) * (sx - ax)
                    dx, dy = bx - ax, by - ay
                    top_left = dy < 0 or (dy == 0 and dx > 0)
                    if not (e > 0 or (e == 0 and top_left)):
                        ok = False
                        break
                if ok:
                    covered.add((px, py))
    return sorted(covered)


def clip_near(poly):
    """Sutherland-Hodgman against z <= w in homogeneous coordinates."""
    out = []
    n = len(poly)
    for i in range(n):
        a, b = poly[i], poly[(i + 1) % n]
        da, db = a[3] - a[2], b[3] - b[2]
        if da >= 0:
            out.append(a)
        if (da >= 0) != (db >= 0):
            t = da / (da - db)
            out.append(tuple(a[k] + t * (b[k] - a[k]) for k in range(4)))
    return out


def raster_cases():
    cases = []
    # 1. A right triangle over an 8x8 view: pixel (x, y) is covered iff
    #    x + y <= 6 (the hypotenuse is a right edge, so centres on it are out).
    tri = [(-1, -1, F(1, 2), 1), (1, -1, F(1, 2), 1), (-1, 1, F(1, 2), 1)]
    cases.append({"name": "right_triangle_8x8", "w": 8, "h": 8, "tris": [tri], "expect": None})
    # 2. The two halves of a square split along its diagonal: every centre of
    #    the square is covered by exactly one half.
    q = [(-1, -1, F(1, 2), 1), (1, -1, F(1, 2), 1), (1, 1, F(1, 2), 1), (-1, 1, F(1, 2), 1)]
    cases.append({"name": "split_square_lower", "w": 8, "h": 8, "tris": [[q[0], q[1], q[2]]], "expect": None})
    cases.append({"name": "split_square_upper", "w": 8, "h": 8, "tris": [[q[0], q[2], q[3]]], "expect": None})
    # 3. Vertical edges through pixel centres: left edge at x = 2.5 includes
    #    column 2, right edge at x = 5.5 excludes column 5.
    x0, x1 = F(25, 10) / 4 - 1, F(55, 10) / 4 - 1
    rect = [(x0, -1, F(1, 2), 1), (x1, -1, F(1, 2), 1), (x1, 1, F(1, 2), 1), (x0, 1, F(1, 2), 1)]
    cases.append({"name": "left_right_ties_a", "w": 8, "h": 8, "tris": [[rect[0], rect[1], rect[2]]], "expect": None})
    cases.append({"name": "left_right_ties_b", "w": 8, "h": 8, "tris": [[rect[0], rect[2], rect[3]]], "expect": None})
    # 4. A triangle crossing the near plane (z > w at one vertex): coverage of
    #    the clipped quadrilateral.
    cross = [(-1, -1, F(1, 2), 1), (1, -1, F(1, 2), 1), (-1, 1, F(2), 1)]
    cases.append({"name": "near_plane_crossing", "w": 8, "h": 8, "tris": [cross], "clip": True, "expect": None})
    # 5. Sub-pixel triangles: one spans the centre of pixel (0, 0), one
    #    misses every centre.
    hit = [(F(-9, 10), F(-9, 10), F(1, 2), 1), (F(-8, 10), F(-9, 10), F(1, 2), 1), (F(-9, 10), F(-8, 10), F(1, 2), 1)]
    cases.append({"name": "tiny_hit", "w": 8, "h": 8, "tris": [hit], "expect": None})
    miss = [(F(-19, 20), F(-19, 20), F(1, 2), 1), (F(-9, 10), F(-19, 20), F(1, 2), 1),
            (F(-19, 20), F(-9, 10), F(1, 2), 1)]
    cases.append({"name": "tiny_miss", "w": 8, "h": 8, "tris": [miss], "expect": None})
    for c in cases:
        cov = set()
        for t in c["tris"]:
            poly = clip_near(list(t)) if c.get("clip") else list(t)
            cov |= set(coverage([screen(v, c["w"], c["h"]) for v in poly], c["w"], c["h"]))
        c["expect"] = sorted(list(p) for p in cov)
        c["tris"] = [[[float(x) for x in v] for v in t] for t in c["tris"]]
        c.pop("clip", None)
    return cases


# -------------------------------------------------------------------- HiZ

def footprint(u: F, size: int):
    t = u * size - F(1, 2)
    i = math.floor(t)
    a = t - i
    out = []
    if 1 - a != 0:
        out.append(min(max(i, 0), size - 1))
    if a != 0:
        out.append(min(max(i + 1, 0), size - 1))
    return out


def hiz_chain(depth, w, h):
    """HiZ reduce chain (hiz_reduce.comp.glsl:21-31, application.cpp:951-1003)."""
    L = 0
    while (2 << L) <= max(w, h):
        L += 1
    mips = []
    src, sw, sh = depth, w, h
    for i in range(1, L + 1):
        dw, dh = w >> i, h >> i
        mw, mh = max(1, (w >> 1) >> (i - 1)), max(1, (h >> 1) >> (i - 1))
        if dw == 0 or dh == 0:
            mips.append([[0.0] * mw for _ in range(mh)])  # never written: pinned to 0.0
            src, sw, sh = mips[-1], mw, mh
            continue
        out = []
        for y in range(dh):
            row = []
            for x in range(dw):
                xs = footprint(F(2 * x + 1, 2 * dw), sw)
                ys = footprint(F(2 * y + 1, 2 * dh), sh)
                row.append(min(src[yy][xx] for yy in ys for xx in xs))
            out.append(row)
        mips.append(out)
        src, sw, sh = out, dw, dh
    return mips


def hiz_cases():
    cases = []
    for (w, h) in [(4, 4), (5, 3), (8, 2), (11, 7), (6, 1)]:
        # depth value of each texel: distinct dyadic rationals (exact in fp32)
        depth = [[((y * w + x) * 37 % 64) / 64.0 for x in range(w)] for y in range(h)]
        cases.append({"w": w, "h": h, "depth": depth, "mips": hiz_chain(depth, w, h)})
    return cases


# ---------------------------------------------------------------- resolve

def from_linear(c: float) -> float:
    return c * 12.92 if c < 0.0031308 else 1.055 * c ** (1 / 2.4) - 0.055


def unorm8(c: float) -> int:
    c = min(max(c, 0.0), 1.0) * 255.0
    return int(round(c))


def resolve_cases():
    out = []
    for albedo in [(0.8, 0.5, 0.3, 1.0), (1.0, 1.0, 1.0, 1.0), (0.0, 0.002, 0.5, 0.25), (0.18, 0.0031308, 0.9, 0.0)]:
        rgba = [unorm8(from_linear(c)) for c in albedo[:3]] + [unorm8(albedo[3])]
        out.append({"albedo": list(albedo), "rgba8": rgba})
    return out


# ------------------------------------------------------------------- cull

def cull_cases():
    # Identity view-projection: clip = (x, y, z, 1); planes = row3 +/- row_i,
    # normalised, w negated (camera.cpp:70-84).
    planes = [[1, 0, 0, -1], [-1, 0, 0, -1], [0, 1, 0, -1], [0, -1, 0, -1], [0, 0, 1, -1], [0, 0, -1, -1]]
    cases = []
    # box exactly touching the x = 1 plane from inside: -radius > distance is false
    cases.append({"name": "face_on_plane", "center": [1.5, 0, 0.5], "extents": [0.5, 0.1, 0.1], "frustum": True})
    cases.append({"name": "just_outside", "center": [1.75, 0, 0.5], "extents": [0.5, 0.1, 0.1], "frustum": False})
    cases.append({"name": "inside", "center": [0, 0, 0.5], "extents": [0.1, 0.1, 0.1], "frustum": True})
    # Occlusion: 64x64 view, pyramid mip0 32x32; the box projects to
    # uv [0.45, 0.55]: width = 0.1 * 32 = 3.2 -> level floor(log2 3.2) = 1;
    # visible iff the level-1 depth < max z = 0.6.
    occl = {"w": 64, "h": 64, "center": [0, 0, 0.5], "extents": [0.1, 0.1, 0.1],
            "cases": [{"mip1_depth": 0.7, "visible": False}, {"mip1_depth": 0.5, "visible": True},
                      {"mip1_depth": 0.6, "visible": False}]}
    return {"planes": planes, "boxes": cases, "occlusion": occl}


def main():
    (HERE / "kat_raster.json").write_text(json.dumps(raster_cases(), indent=1))
    (HERE / "kat_hiz.json").write_text(json.dumps(hiz_cases()))
    (HERE / "kat_resolve.json").write_text(json.dumps(resolve_cases(), indent=1))
    (HERE / "kat_cull.json").write_text(json.dumps(cull_cases(), indent=1))


if __name__ == "__main__":
    main()
