"""ctypes binding of the CPU oracle (oracle.c).  TEST INFRASTRUCTURE ONLY:
imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the checker, never by the product package.

Parity status: the oracle is pinned by hand-derived known-answer cases only;
parity with the reference renderer's own execution is unpinned (it needs a
Vulkan mesh-shader device, which does not exist here).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

CULL_FRUSTUM = 1 << 0
CULL_OCCLUSION = 1 << 1
CULL_TWO_PASS = 1 << 2
CULL_CONE = 1 << 3
RESOLVE_FLAT = 1 << 4
RESOLVE_TEXTURED = 1 << 5
BUILD_PYRAMID = 1 << 6
CULL_OCCLUSION_FINE = 1 << 7


class OrcPrimitive(C.Structure):
    _fields_ = [("vertex_indices", C.c_void_p), ("primitive_indices", C.c_void_p), ("vertices", C.c_void_p),
                ("meshlets", C.c_void_p), ("aabb_extents", C.c_float * 3), ("aabb_center", C.c_float * 3),
                ("meshlet_count", C.c_uint32), ("material_index", C.c_uint32), ("cones", C.c_void_p)]


class OrcTexture(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32),
                ("row_pitch", C.c_uint32)]


class OrcScene(C.Structure):
    _fields_ = [("draws", C.c_void_p), ("draw_count", C.c_uint32), ("transforms", C.c_void_p),
                ("primitives", C.c_void_p), ("materials", C.c_void_p), ("textures", C.c_void_p),
                ("texture_count", C.c_uint32)]


class OrcPyramid(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("levels", C.c_uint32),
                ("view_width", C.c_uint32), ("view_height", C.c_uint32)]


class OrcWorld(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("node_count", C.c_uint32), ("child_count", C.c_uint32),
                ("children", C.c_void_p), ("roots", C.c_void_p), ("root_count", C.c_uint32),
                ("mesh_count", C.c_uint32), ("mesh_offsets", C.c_void_p), ("mesh_primitives", C.c_void_p),
                ("primitive_meshlet_counts", C.c_void_p), ("primitive_count", C.c_uint32),
                ("sampler_count", C.c_uint32), ("samplers", C.c_void_p), ("channels", C.c_void_p),
                ("channel_count", C.c_uint32), ("pad_", C.c_uint32)]


class OrcAnimSampler(C.Structure):
    _fields_ = [("input", C.c_void_p), ("output", C.c_void_p), ("input_count", C.c_uint32),
                ("output_count", C.c_uint32), ("interpolation", C.c_uint32), ("components", C.c_uint32)]


_lib = None
_ref = None
REF_LIB = HERE / "_ref" / "libvkgv_ref.so"


def reference_sources() -> Path | None:
    """The reference's source tree when it is present on this machine (the
    reference build of _ref/ needs its shaders/ directory); None elsewhere."""
    root = Path(os.environ.get("VKGV_REFERENCE", "/root/reference"))
    return root if (root / "shaders" / "common.h.glsl").exists() else None


def build_ref() -> Path | None:
    """Compiles the reference's shared GLSL headers in their C++ mode into
    _ref/libvkgv_ref.so (oracle/Makefile `ref`).  Returns None when the
    reference sources are absent, or the library already built earlier."""
    src = reference_sources()
    if src is None:
        return REF_LIB if REF_LIB.exists() else None
    res = subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={src}"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference header build failed:\n{res.stdout}\n{res.stderr}")
    return REF_LIB


def load_ref() -> C.CDLL | None:
    """The reference-header library (see build_ref), or None if unbuilt."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists() and build_ref() is None:
            return None
        lib = C.CDLL(str(REF_LIB))
        U32 = C.c_uint32
        lib.ref_layout_count.restype = U32
        lib.ref_layout_name.restype = C.c_char_p
        lib.ref_layout_name.argtypes = [U32]
        lib.ref_layout_value.restype = U32
        lib.ref_layout_value.argtypes = [U32]
        lib.ref_pack_visbuffer.restype = U32
        lib.ref_pack_visbuffer.argtypes = [U32, U32]
        lib.ref_unpack_visbuffer.argtypes = [U32, C.POINTER(U32), C.POINTER(U32)]
        lib.ref_from_linear.restype = C.c_float
        lib.ref_from_linear.argtypes = [C.c_float]
        lib.ref_to_linear.restype = C.c_float
        lib.ref_to_linear.argtypes = [C.c_float]
        lib.ref_from_linear4.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_to_linear4.argtypes = [C.c_void_p, C.c_void_p]
        _ref = lib
    return _ref


def ref_layout(lib) -> dict[str, int]:
    return {lib.ref_layout_name(i).decode(): int(lib.ref_layout_value(i)) for i in range(lib.ref_layout_count())}


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, no fast-math)."""
    res = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        P = C.c_void_p
        U32 = C.c_uint32
        lib.orc_set_threads.argtypes = [C.c_int]
        lib.orc_get_threads.restype = C.c_int
        lib.orc_pyramid_levels.restype = U32
        lib.orc_pyramid_levels.argtypes = [U32, U32]
        lib.orc_pyramid_floats.restype = C.c_uint64
        lib.orc_pyramid_floats.argtypes = [U32, U32]
        lib.orc_cull.argtypes = [P, P, P, U32, U32, P, U32, P, P, P, P]
        lib.orc_raster.argtypes = [P, P, U32, U32, P, U32, P]
        lib.orc_hiz.argtypes = [P, U32, U32, P]
        lib.orc_resolve.argtypes = [P, P, U32, U32, P, U32, P, P]
        lib.orc_frame.argtypes = [P, P, U32, U32, P, U32, P, P, P, P, P, P]
        lib.orc_motion.argtypes = [P, P, U32, U32, P, P]
        lib.orc_world_transforms.restype = C.c_int64
        lib.orc_world_transforms.argtypes = [P, C.c_float, P, U32]
        lib.orc_world_draws.restype = C.c_int64
        lib.orc_world_draws.argtypes = [P, P, C.c_uint64]
        lib.orc_anim_sample.argtypes = [P, C.c_float, U32, P]
        lib.orc_slerp.argtypes = [P, P, C.c_float, P]
        lib.orc_trs_matrix.argtypes = [P, P, P, P]
        lib.orc_sin_series.restype = C.c_float
        lib.orc_sin_series.argtypes = [C.c_float]
        lib.orc_asin_series.restype = C.c_float
        lib.orc_asin_series.argtypes = [C.c_float]
        lib.orc_decode_bc.argtypes = [U32, P, U32, U32, P]
        lib.orc_decode_bc6h.argtypes = [P, U32, U32, C.c_int, P]
        lib.orc_jpeg_idct.argtypes = [P, U32, U32, P]
        lib.orc_jpeg_color.argtypes = [P, P, P, P, P, P, U32, U32, U32, U32, P]
        lib.orc_half_rn.restype = C.c_uint16
        lib.orc_half_rn.argtypes = [C.c_float]
        lib.orc_from_linear.restype = C.c_float
        lib.orc_from_linear.argtypes = [C.c_float]
        lib.orc_to_linear.restype = C.c_float
        lib.orc_to_linear.argtypes = [C.c_float]
        lib.orc_unorm8.restype = U32
        lib.orc_unorm8.argtypes = [C.c_float]
        lib.orc_raster_triangle.argtypes = [P, P, P, U32, U32, U32, P]
        lib.orc_min_sample.restype = C.c_float
        lib.orc_min_sample.argtypes = [P, U32, U32, C.c_float, C.c_float]
        lib.orc_frustum_visible.restype = C.c_int
        lib.orc_frustum_visible.argtypes = [P, P, P]
        _lib = lib
    return _lib


def set_threads(n: int) -> None:
    load().orc_set_threads(int(n))


def _addr(a: np.ndarray) -> int:
    return int(a.ctypes.data)


class OracleScene:
    """orc_scene over the host arrays of a HostScene (kept alive here)."""

    def __init__(self, host):
        self.host = host
        self._keep = []
        prims = (OrcPrimitive * len(host.meshes))()
        for p, m in enumerate(host.meshes):
            arrs = [np.ascontiguousarray(m.vertex_indices), np.ascontiguousarray(m.primitive_indices),
                    np.ascontiguousarray(m.vertices), np.ascontiguousarray(m.meshlets)]
            self._keep += arrs
            prims[p].vertex_indices, prims[p].primitive_indices, prims[p].vertices, prims[p].meshlets = map(_addr, arrs)
            prims[p].aabb_extents[:] = [float(x) for x in m.aabb_extents]
            prims[p].aabb_center[:] = [float(x) for x in m.aabb_center]
            prims[p].meshlet_count = m.meshlet_count
            prims[p].material_index = host.prim_materials[p]
            if m.cones is not None and m.cones.size:
                cones = np.ascontiguousarray(m.cones)
                self._keep.append(cones)
                prims[p].cones = _addr(cones)
        self.prims = prims
        self.draws = np.ascontiguousarray(host.draws, np.uint32)
        self.transforms = np.ascontiguousarray(host.transforms, np.float32)
        self.materials = np.ascontiguousarray(host.materials)
        texs = (OrcTexture * max(1, len(host.textures)))()
        for i, t in enumerate(host.textures):
            d = np.ascontiguousarray(t.data)
            self._keep.append(d)
            texs[i].data = _addr(d)
            texs[i].width, texs[i].height, texs[i].format, texs[i].row_pitch = t.width, t.height, t.format, t.width
        self.texs = texs
        self.s = OrcScene(draws=_addr(self.draws), draw_count=host.draw_count, transforms=_addr(self.transforms),
                          primitives=C.addressof(prims), materials=_addr(self.materials),
                          textures=C.addressof(texs), texture_count=len(host.textures))

    @property
    def ptr(self):
        return C.addressof(self.s)


def pyramid_floats(w: int, h: int) -> int:
    return int(load().orc_pyramid_floats(w, h))


def pyramid_levels(w: int, h: int) -> int:
    return int(load().orc_pyramid_levels(w, h))


def cull(os_: OracleScene, cam, w: int, h: int, flags: int, pass_: int = 1, pyramid: np.ndarray | None = None,
         candidates: np.ndarray | None = None):
    """Returns (survivors, occlusion_rejects) as uint32 arrays."""
    lib = load()
    n = os_.host.draw_count if candidates is None else int(candidates.size)
    surv = np.zeros(max(1, n), np.uint32)
    rej = np.zeros(max(1, n), np.uint32)
    ns, nr = C.c_uint32(), C.c_uint32()
    pyr = None
    if pyramid is not None:
        pyramid = np.ascontiguousarray(pyramid, np.float32)
        pyr = OrcPyramid(_addr(pyramid), w >> 1, h >> 1, pyramid_levels(w, h), w, h)
    cand = None if candidates is None else np.ascontiguousarray(candidates, np.uint32)
    lib.orc_cull(os_.ptr, C.addressof(cam), C.addressof(pyr) if pyr is not None else None, flags, pass_,
                 _addr(cand) if cand is not None else None, n, _addr(surv), C.addressof(ns), _addr(rej),
                 C.addressof(nr))
    return surv[: ns.value].copy(), rej[: nr.value].copy()


def raster(os_: OracleScene, cam, w: int, h: int, draws: np.ndarray, depth_id: np.ndarray | None = None):
    lib = load()
    draws = np.ascontiguousarray(draws, np.uint32)
    if depth_id is None:
        depth_id = np.zeros(w * h, np.uint64)
    lib.orc_raster(os_.ptr, C.addressof(cam), w, h, _addr(draws) if draws.size else None, draws.size,
                   _addr(depth_id))
    return depth_id


def hiz(depth_id: np.ndarray, w: int, h: int) -> np.ndarray:
    pyr = np.zeros(max(1, pyramid_floats(w, h)), np.float32)
    load().orc_hiz(_addr(np.ascontiguousarray(depth_id, np.uint64)), w, h, _addr(pyr))
    return pyr


def resolve(os_: OracleScene, cam, w: int, h: int, depth_id: np.ndarray, textured: bool = False):
    ids = np.zeros(w * h, np.uint32)
    rgba = np.zeros(w * h, np.uint32)
    load().orc_resolve(os_.ptr, C.addressof(cam), w, h, _addr(np.ascontiguousarray(depth_id, np.uint64)),
                       1 if textured else 0, _addr(ids), _addr(rgba))
    return ids, rgba


def motion(os_: OracleScene, cam, w: int, h: int, depth_id: np.ndarray) -> np.ndarray:
    """Motion vectors of the visible fragments of a finished depth_id image:
    uint32[w*h], two binary16 per pixel (x low), 0 where nothing was drawn."""
    depth = np.ascontiguousarray(depth_id, np.uint64).reshape(-1)
    if depth.size != w * h:
        raise ValueError(f"depth_id has {depth.size} pixels, expected {w * h}")
    out = np.zeros(w * h, np.uint32)
    load().orc_motion(os_.ptr, C.addressof(cam), w, h, _addr(depth), _addr(out))
    return out


def half_rn(v: float) -> int:
    """binary32 -> binary16 bits, round to nearest even."""
    return int(load().orc_half_rn(v))


def frame(os_: OracleScene, cam, w: int, h: int, flags: int, prev_pyramid: np.ndarray | None = None):
    """Whole frame; returns dict with depth_id, ids, rgba, pyramid, survivors."""
    lib = load()
    depth = np.zeros(w * h, np.uint64)
    ids = np.zeros(w * h, np.uint32)
    rgba = np.zeros(w * h, np.uint32)
    pyr = np.zeros(max(1, pyramid_floats(w, h)), np.float32)
    surv = np.zeros(max(1, os_.host.draw_count), np.uint32)
    ns = C.c_uint32()
    prev = None
    if prev_pyramid is not None:
        prev_pyramid = np.ascontiguousarray(prev_pyramid, np.float32)
        prev = OrcPyramid(_addr(prev_pyramid), w >> 1, h >> 1, pyramid_levels(w, h), w, h)
    lib.orc_frame(os_.ptr, C.addressof(cam), w, h, C.addressof(prev) if prev is not None else None, flags,
                  _addr(depth), _addr(ids), _addr(rgba), _addr(pyr), _addr(surv), C.addressof(ns))
    return {"depth_id": depth, "ids": ids, "rgba": rgba, "pyramid": pyr, "survivors": surv[: ns.value].copy()}


def raster_triangle(v0, v1, v2, tri_id: int, w: int, h: int, depth_id: np.ndarray | None = None):
    if depth_id is None:
        depth_id = np.zeros(w * h, np.uint64)
    a = [np.ascontiguousarray(v, np.float32) for v in (v0, v1, v2)]
    load().orc_raster_triangle(_addr(a[0]), _addr(a[1]), _addr(a[2]), tri_id, w, h, _addr(depth_id))
    return depth_id


def min_sample(img: np.ndarray, u: float, v: float) -> float:
    img = np.ascontiguousarray(img, np.float32)
    return float(load().orc_min_sample(_addr(img), img.shape[1], img.shape[0], u, v))


def frustum_visible(center, extents, planes) -> bool:
    c = np.ascontiguousarray(center, np.float32)
    e = np.ascontiguousarray(extents, np.float32)
    p = np.ascontiguousarray(planes, np.float32).reshape(24)
    return bool(load().orc_frustum_visible(_addr(c), _addr(e), _addr(p)))


class OrcDiffScene(C.Structure):
    _fields_ = [("meshlets", C.c_void_p), ("vertex_indices", C.c_void_p), ("tri_indices", C.c_void_p),
                ("positions", C.c_void_p), ("colors", C.c_void_p), ("uvs", C.c_void_p), ("texture", C.c_void_p),
                ("tex_w", C.c_uint32), ("tex_h", C.c_uint32), ("albedo", C.c_double * 3),
                ("uv_offset", C.c_double * 2), ("uv_scale", C.c_double * 2), ("uv_rotation", C.c_double)]


def diff_f64(mesh, positions, colors, uvs, texture, vp16, w: int, h: int, ids: np.ndarray,
             target: np.ndarray | None = None, scale: float = 1.0, albedo=(1.0, 1.0, 1.0), uv_offset=(0.0, 0.0),
             uv_scale=(1.0, 1.0), uv_rotation: float = 0.0, want_rgb=False, want_grads=False,
             cells: np.ndarray | None = None, freeze: np.ndarray | None = None,
             margin: np.ndarray | None = None):
    """float64 shading/loss/gradients at fixed visibility `ids` (uint32 per
    pixel).  Parameters are converted to float64.  Returns (loss, rgb or None,
    (gpos, gcol, gtex) or None).  `cells`, an int32 array of 2*w*h, receives
    each pixel's unwrapped bilinear cell (INT32_MIN for empty pixels).
    `freeze` (int32, 2*w*h, as `cells` reports them) holds each pixel's
    bilinear cell fixed (orc_diff_f64_frozen).  `margin` (float64, w*h)
    receives each pixel's distance in texels to the nearest texel-centre
    line (-1 for empty pixels)."""
    lib = load()
    if not hasattr(lib.orc_diff_f64_frozen, "_typed"):
        lib.orc_diff_f64_frozen.restype = C.c_double
        lib.orc_diff_f64_frozen.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                            C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.orc_diff_f64_frozen._typed = True
    keep = [np.ascontiguousarray(mesh.meshlets), np.ascontiguousarray(mesh.vertex_indices),
            np.ascontiguousarray(mesh.primitive_indices), np.ascontiguousarray(positions, np.float64),
            np.ascontiguousarray(colors, np.float64), np.ascontiguousarray(uvs, np.float64),
            np.ascontiguousarray(texture, np.float64)]
    s = OrcDiffScene(meshlets=_addr(keep[0]), vertex_indices=_addr(keep[1]), tri_indices=_addr(keep[2]),
                     positions=_addr(keep[3]), colors=_addr(keep[4]), uvs=_addr(keep[5]), texture=_addr(keep[6]),
                     tex_w=int(np.asarray(texture).shape[1]), tex_h=int(np.asarray(texture).shape[0]),
                     uv_rotation=float(uv_rotation))
    s.albedo[:] = list(albedo)
    s.uv_offset[:] = list(uv_offset)
    s.uv_scale[:] = list(uv_scale)
    vp = np.ascontiguousarray(vp16, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    tgt = None if target is None else np.ascontiguousarray(target, np.float32)
    rgb = np.zeros(w * h * 3, np.float64) if want_rgb else None
    grads = None
    if want_grads:
        grads = (np.zeros(keep[3].size), np.zeros(keep[4].size), np.zeros(keep[6].size))
    frz = None
    if freeze is not None:
        frz = np.ascontiguousarray(freeze, np.int32)
        if frz.size != 2 * w * h:
            raise ValueError("freeze needs 2 int32 per pixel")
    loss = lib.orc_diff_f64_frozen(C.addressof(s), _addr(vp), w, h, _addr(ids),
                                   _addr(tgt) if tgt is not None else None, float(scale),
                                   _addr(rgb) if rgb is not None else None,
                                   *(tuple(_addr(g) for g in grads) if grads else (None, None, None)),
                                   _cells_addr(cells, w, h), _addr(frz) if frz is not None else None,
                                   _margin_addr(margin, w, h))
    return float(loss), rgb, grads


def _margin_addr(margin, w, h):
    if margin is None:
        return None
    if margin.dtype != np.float64 or margin.size != w * h or not margin.flags.c_contiguous:
        raise ValueError("margin must be a contiguous float64 array of w*h")
    return _addr(margin)


def _cells_addr(cells, w, h):
    if cells is None:
        return None
    if cells.dtype != np.int32 or cells.size != 2 * w * h or not cells.flags.c_contiguous:
        raise ValueError("cells must be a contiguous int32 array of 2*w*h")
    return _addr(cells)


def from_linear(c: float) -> float:
    return float(load().orc_from_linear(c))


def unorm8(c: float) -> int:
    return int(load().orc_unorm8(c))


# ------------------------------------------------------------------ world

def _orc_world(host) -> OrcWorld:
    """The oracle's orc_world over a HostWorld's arrays (same layout as the
    library's vkgv_world_desc)."""
    return OrcWorld(**host.desc_fields())


def world_transforms(host, animation_time: float) -> np.ndarray:
    """World::updateTransformBuffer: (T, 16) float32, column-major."""
    lib = load()
    w = _orc_world(host)
    n = lib.orc_world_transforms(C.addressof(w), animation_time, None, 0)
    if n < 0:
        raise ValueError("node tree deeper than 64")
    out = np.zeros((max(1, n), 16), np.float32)
    lib.orc_world_transforms(C.addressof(w), animation_time, _addr(out), n)
    return out[:n]


def world_draws(host) -> np.ndarray:
    """World::rebuildDrawBuffer: (D, 3) uint32 {primitive, meshlet, transform}."""
    lib = load()
    w = _orc_world(host)
    n = lib.orc_world_draws(C.addressof(w), None, 0)
    if n < 0:
        raise ValueError("node tree deeper than 64")
    out = np.zeros((max(1, n), 3), np.uint32)
    lib.orc_world_draws(C.addressof(w), _addr(out), n)
    return out[:n]


def anim_sample(times: np.ndarray, values: np.ndarray, interpolation: int, t: float, path: int) -> np.ndarray:
    """AnimationSampler::sample of one sampler (values: (output_count, components))."""
    times = np.ascontiguousarray(times, np.float32)
    values = np.ascontiguousarray(values, np.float32)
    s = OrcAnimSampler(times.ctypes.data, values.ctypes.data, times.size, values.shape[0], interpolation,
                       values.shape[1])
    out = np.zeros(4, np.float32)
    load().orc_anim_sample(C.addressof(s), t, path, _addr(out))
    return out[: values.shape[1]]


def slerp(a, b, t: float) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.zeros(4, np.float32)
    load().orc_slerp(_addr(a), _addr(b), t, _addr(out))
    return out


def trs_matrix(t, q, s) -> np.ndarray:
    t = np.ascontiguousarray(t, np.float32)
    q = np.ascontiguousarray(q, np.float32)
    s = np.ascontiguousarray(s, np.float32)
    out = np.zeros(16, np.float32)
    load().orc_trs_matrix(_addr(t), _addr(q), _addr(s), _addr(out))
    return out


def sin_series(x: float) -> float:
    return float(load().orc_sin_series(x))


def asin_series(z: float) -> float:
    return float(load().orc_asin_series(z))


def decode_bc(fmt: int, blocks: np.ndarray, w: int, h: int) -> np.ndarray:
    """BC1-BC5 blocks -> uint32 RGBA8 texels (h, w)."""
    blocks = np.ascontiguousarray(blocks, np.uint8)
    need = ((w + 3) // 4) * ((h + 3) // 4) * (8 if fmt in (1, 4, 6) else 16)
    if blocks.size < need:
        raise ValueError(f"{blocks.size} block bytes, {need} needed")
    out = np.zeros(w * h, np.uint32)
    load().orc_decode_bc(fmt, _addr(blocks), w, h, _addr(out))
    return out.reshape(h, w)


def decode_bc6h(blocks: np.ndarray, w: int, h: int, signed: bool) -> np.ndarray:
    """BC6H blocks -> (h, w, 3) uint16 binary16 bits (SF16 when `signed`)."""
    blocks = np.ascontiguousarray(blocks, np.uint8)
    need = ((w + 3) // 4) * ((h + 3) // 4) * 16
    if blocks.size < need:
        raise ValueError(f"{blocks.size} block bytes, {need} needed")
    out = np.zeros(w * h * 3, np.uint16)
    load().orc_decode_bc6h(_addr(blocks), w, h, 1 if signed else 0, _addr(out))
    return out.reshape(h, w, 3)


def jpeg_rgba(info, planes) -> np.ndarray:
    """JPEG pixels from its coefficient planes: `info` has width, height,
    components, rgb, hmax, vmax, h, v, blocks_w, blocks_h (as
    vkgv_jpeg_info); planes[c] is (blocks_h * blocks_w * 64) int16.
    Returns (height, width) uint32 RGBA8."""
    lib = load()
    samples, pitch, rx, ry = [], [], [], []
    for c in range(info.components):
        bw, bh = int(info.blocks_w[c]), int(info.blocks_h[c])
        coef = np.ascontiguousarray(planes[c], np.int16)
        assert coef.size == bw * bh * 64
        plane = np.zeros(bw * bh * 64, np.uint8)
        lib.orc_jpeg_idct(_addr(coef), bw, bh, _addr(plane))
        samples.append(plane)
        pitch.append(bw * 8)
        rx.append(int(info.hmax) // int(info.h[c]))
        ry.append(int(info.vmax) // int(info.v[c]))
    while len(samples) < 3:
        samples.append(samples[0])
        pitch.append(0)
        rx.append(1)
        ry.append(1)
    arr = [np.asarray(a, np.uint32) for a in (pitch, rx, ry)]
    out = np.zeros(int(info.width) * int(info.height), np.uint32)
    lib.orc_jpeg_color(_addr(samples[0]), _addr(samples[1]), _addr(samples[2]), _addr(arr[0]), _addr(arr[1]),
                       _addr(arr[2]), int(info.width), int(info.height), int(info.components), int(info.rgb),
                       _addr(out))
    return out.reshape(int(info.height), int(info.width))
