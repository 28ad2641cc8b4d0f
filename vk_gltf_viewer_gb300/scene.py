"""Host-side scene assembly in the renderer's buffer layout.

Meshes, meshlets and cameras come from the C++ producers in libvkgv
(scene.cpp); this module arranges them into the draw list, transform, material
and texture buffers the reference builds in World::rebuildDrawBuffer
(src/vk_gltf_viewer/world.cpp:230-293) and uploads them as device buffers whose
addresses fill the glsl::Primitive pointers.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

MESHLET_DTYPE = np.dtype({"names": ["vertex_offset", "triangle_offset", "vertex_count", "triangle_count", "pad",
                                    "aabb_extents", "aabb_center"],
                          "formats": ["<u4", "<u4", "u1", "u1", ("u1", 2), ("<f4", 3), ("<f4", 3)],
                          "offsets": [0, 4, 8, 9, 10, 12, 24], "itemsize": 36})
VERTEX_DTYPE = np.dtype({"names": ["position", "color", "normal", "pad", "uv"],
                         "formats": [("<f4", 3), ("u1", 4), ("u1", 3), "u1", ("<u2", 2)],
                         "offsets": [0, 12, 16, 19, 20], "itemsize": 24})
CONE_DTYPE = np.dtype({"names": ["center", "radius", "axis", "cutoff"],
                       "formats": [("<f4", 3), "<f4", ("<f4", 3), "<f4"],
                       "offsets": [0, 12, 16, 28], "itemsize": 32})
MATERIAL_DTYPE = np.dtype({"names": ["albedo_factor", "albedo_index", "uv_offset", "uv_scale", "uv_rotation",
                                     "alpha_cutoff", "double_sided"],
                           "formats": [("<f4", 4), "<u4", ("<f4", 2), ("<f4", 2), "<f4", "<f4", "<u4"],
                           "offsets": [0, 16, 20, 28, 36, 40, 44], "itemsize": 48})


@dataclass
class Mesh:
    """One primitive's streams (copied out of the C++ producer)."""
    vertices: np.ndarray          # VERTEX_DTYPE
    positions: np.ndarray         # (V, 3) float32 (stored positions)
    uvs: np.ndarray | None        # (V, 2) float32
    indices: np.ndarray           # (T, 3) uint32
    meshlets: np.ndarray          # MESHLET_DTYPE
    vertex_indices: np.ndarray    # uint32
    primitive_indices: np.ndarray  # uint8
    aabb_extents: np.ndarray
    aabb_center: np.ndarray
    position_scale: float = 1.0
    cones: np.ndarray | None = None  # CONE_DTYPE, one per meshlet

    @property
    def meshlet_count(self) -> int:
        return int(self.meshlets.shape[0])

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])


def _copy(ptr, n: int, dtype) -> np.ndarray:
    dtype = np.dtype(dtype)
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    raw = C.string_at(ptr, n * dtype.itemsize)
    return np.frombuffer(raw, dtype=dtype, count=n).copy()


def _mesh_from_handle(h, max_vertices: int = 64, max_triangles: int = 124, owned: bool = True) -> Mesh:
    """Copies a mesh handle's streams out.  An owned handle is meshletised
    here and freed; a borrowed one (an imported asset's) is read as is."""
    lib = abi.load()
    if not h:
        raise abi.VkgvError(abi.INVALID_ARG, "mesh producer failed")
    try:
        if owned:
            abi.check(lib.vkgv_mesh_build_meshlets(h, max_vertices, max_triangles))
        info = abi.MeshInfo()
        abi.check(lib.vkgv_mesh_get_info(h, C.byref(info)))
        nv, nt = info.vertex_count, info.triangle_count
        return Mesh(
            vertices=_copy(C.cast(info.vertices, C.c_void_p).value, nv, VERTEX_DTYPE),
            positions=_copy(C.cast(info.positions, C.c_void_p).value, nv * 3, np.float32).reshape(nv, 3),
            uvs=(_copy(C.cast(info.uvs, C.c_void_p).value, nv * 2, np.float32).reshape(nv, 2)
                 if info.uvs else None),
            indices=_copy(C.cast(info.indices, C.c_void_p).value, nt * 3, np.uint32).reshape(nt, 3),
            meshlets=_copy(C.cast(info.meshlets, C.c_void_p).value, info.meshlet_count, MESHLET_DTYPE),
            vertex_indices=_copy(C.cast(info.vertex_indices, C.c_void_p).value, info.vertex_index_count, np.uint32),
            primitive_indices=_copy(C.cast(info.primitive_indices, C.c_void_p).value,
                                    info.primitive_index_bytes, np.uint8),
            aabb_extents=np.array(info.aabb_extents[:], np.float32),
            aabb_center=np.array(info.aabb_center[:], np.float32),
            position_scale=float(info.position_scale),
            cones=_copy(C.cast(info.cones, C.c_void_p).value, info.meshlet_count, CONE_DTYPE),
        )
    finally:
        if owned:
            lib.vkgv_mesh_free(h)


def icosphere(level: int, displace: float = 0.0, seed: int = 0, rgba: np.ndarray | None = None) -> Mesh:
    lib = abi.load()
    h = lib.vkgv_mesh_icosphere(level)
    if not h:
        raise abi.VkgvError(abi.INVALID_ARG, f"icosphere level {level}")
    if displace:
        abi.check(lib.vkgv_mesh_displace(h, displace, seed))
    if rgba is not None:
        rgba = np.ascontiguousarray(rgba, np.float32)
        abi.check(lib.vkgv_mesh_set_attributes(h, rgba.ctypes.data_as(C.POINTER(C.c_float)), None))
    return _mesh_from_handle(h)


def torus(R: float = 1.0, r: float = 0.35, seg_major: int = 200, seg_minor: int = 100, noise_amp: float = 0.05,
          seed: int = 1, quantize: bool = True) -> Mesh:
    h = abi.load().vkgv_mesh_torus(R, r, seg_major, seg_minor, noise_amp, seed, 1 if quantize else 0)
    return _mesh_from_handle(h)


def mesh_from_arrays(positions: np.ndarray, indices: np.ndarray, max_vertices: int = 64,
                     max_triangles: int = 124) -> Mesh:
    p = np.ascontiguousarray(positions, np.float32)
    i = np.ascontiguousarray(indices, np.uint32)
    h = abi.load().vkgv_mesh_from_arrays(p.ctypes.data_as(C.POINTER(C.c_float)), p.shape[0],
                                         i.ctypes.data_as(C.POINTER(C.c_uint32)), i.shape[0])
    return _mesh_from_handle(h, max_vertices, max_triangles)


# ------------------------------------------------------------------ matrices

def mat_translate(t) -> np.ndarray:
    m = np.eye(4, dtype=np.float64)
    m[:3, 3] = t
    return m


def mat_rotate_y(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4, dtype=np.float64)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def mat_scale(s) -> np.ndarray:
    m = np.eye(4, dtype=np.float64)
    m[0, 0], m[1, 1], m[2, 2] = (s, s, s) if np.isscalar(s) else s
    return m


def to_column_major(m: np.ndarray) -> np.ndarray:
    """4x4 row-major math matrix -> 16 floats, column-major (glm layout)."""
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(16), np.float32)


# ------------------------------------------------------------------- scenes

@dataclass
class Texture:
    data: np.ndarray      # (H, W, 4) uint8 or (H, W, 3) float32
    format: int

    @property
    def width(self) -> int:
        return int(self.data.shape[1])

    @property
    def height(self) -> int:
        return int(self.data.shape[0])


@dataclass
class HostScene:
    """Host copy of every scene buffer (the layout of vkgv.h)."""
    meshes: list[Mesh]
    prim_materials: list[int]
    materials: np.ndarray          # MATERIAL_DTYPE
    transforms: np.ndarray         # (N, 16) float32, column-major
    node_meshes: list[list[int]]   # primitives drawn by each node, in draw order
    textures: list[Texture] = field(default_factory=list)
    draws: np.ndarray | None = None  # (D, 3) uint32

    def __post_init__(self):
        if self.draws is None:
            self.draws = build_draws(self.meshes, self.node_meshes)

    @property
    def draw_count(self) -> int:
        return int(self.draws.shape[0])

    @property
    def triangle_count(self) -> int:
        return int(sum(self.meshes[p].triangle_count for prims in self.node_meshes for p in prims))


def build_draws(meshes: list[Mesh], node_meshes: list[list[int]]) -> np.ndarray:
    """One MeshletDraw per (node, primitive, meshlet) in node -> primitive ->
    meshlet order (world.cpp:245-262); the transform index counts nodes."""
    parts = []
    for t, prims in enumerate(node_meshes):
        for p in prims:
            n = meshes[p].meshlet_count
            d = np.empty((n, 3), np.uint32)
            d[:, 0] = p
            d[:, 1] = np.arange(n, dtype=np.uint32)
            d[:, 2] = t
            parts.append(d)
    if not parts:
        return np.zeros((0, 3), np.uint32)
    return np.ascontiguousarray(np.concatenate(parts))


def make_material(albedo=(1.0, 1.0, 1.0, 1.0), albedo_index=abi.INVALID_HANDLE, uv_offset=(0.0, 0.0),
                  uv_scale=(1.0, 1.0), uv_rotation=0.0, alpha_cutoff=0.5, double_sided=False) -> np.ndarray:
    m = np.zeros(1, MATERIAL_DTYPE)
    m["albedo_factor"] = albedo
    m["albedo_index"] = albedo_index
    m["uv_offset"] = uv_offset
    m["uv_scale"] = uv_scale
    m["uv_rotation"] = uv_rotation
    m["alpha_cutoff"] = alpha_cutoff
    m["double_sided"] = 1 if double_sided else 0
    return m


def default_material() -> np.ndarray:
    """Material 0: the glTF default (assets.cpp:486-492)."""
    return make_material()


def scene_icosphere(level: int = 6, albedo=(0.8, 0.5, 0.3, 1.0)) -> HostScene:
    """Single icosphere node with one material of constant base colour
    (glTF material index 0 stored at 1, assets.cpp:292-294)."""
    mesh = icosphere(level)
    mats = np.concatenate([default_material(), make_material(albedo)])
    return HostScene(meshes=[mesh], prim_materials=[1], materials=mats,
                     transforms=to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])


GRID = (16, 16, 8)   # x, z (long axes) and y (layers)
SPACING = 2.5


def grid_centre() -> np.ndarray:
    gx, gz, gy = GRID
    return np.array([(gx - 1) * SPACING / 2, (gy - 1) * SPACING / 2, (gz - 1) * SPACING / 2])


def scene_torus_grid(seed: int = 7, texture_size: int = 2048, grid=GRID, tex_seed: int = 11) -> HostScene:
    """Seeded displaced torus (KHR_mesh_quantization streams) instanced on a
    16 x 16 x 8 grid (spacing 2.5) with random yaw, one RGBA8 noise texture
    with a KHR_texture_transform scale of 4."""
    mesh = torus(seed=seed)
    rng = np.random.default_rng(seed)
    gx, gz, gy = grid
    transforms = []
    for k in range(gy):
        for j in range(gz):
            for i in range(gx):
                yaw = rng.uniform(0, 2 * math.pi)
                m = mat_translate((i * SPACING, k * SPACING, j * SPACING)) @ mat_rotate_y(yaw) @ mat_scale(
                    mesh.position_scale)
                transforms.append(to_column_major(m))
    transforms = np.stack(transforms)
    textures = []
    albedo_index = abi.INVALID_HANDLE
    if texture_size:
        trng = np.random.default_rng(tex_seed)
        tex = trng.integers(0, 256, size=(texture_size, texture_size, 4), dtype=np.uint8)
        tex[..., 3] = 255
        textures.append(Texture(tex, abi.TEXTURE_RGBA8))
        albedo_index = 0
    mats = np.concatenate([default_material(), make_material((1.0, 1.0, 1.0, 1.0), albedo_index=albedo_index,
                                                             uv_scale=(4.0, 4.0))])
    return HostScene(meshes=[mesh], prim_materials=[1], materials=mats, transforms=transforms,
                     node_meshes=[[0] for _ in range(transforms.shape[0])], textures=textures)


# ------------------------------------------------------------------ cameras

def camera(eye, target, up=(0.0, 1.0, 0.0), fovy_deg: float = 60.0, aspect: float = 16 / 9,
           znear: float = 0.1, zfar: float = 1000.0, prev: abi.Camera | None = None) -> abi.Camera:
    """Camera buffer after one update (camera.cpp:170-193).  With `prev`, the
    previous matrices come from it; otherwise current and previous match."""
    cam = abi.Camera()
    if prev is not None:
        C.memmove(C.byref(cam), C.byref(prev), C.sizeof(cam))
    e = (C.c_float * 3)(*eye)
    t = (C.c_float * 3)(*target)
    u = (C.c_float * 3)(*up)
    abi.check(abi.load().vkgv_camera_update(C.byref(cam), e, t, u, math.radians(fovy_deg), aspect, znear, zfar))
    if prev is None:
        # a static camera: the previous frame saw the same matrices
        abi.check(abi.load().vkgv_camera_update(C.byref(cam), e, t, u, math.radians(fovy_deg), aspect, znear, zfar))
    return cam


def safe_up(eye, target) -> tuple:
    d = np.asarray(target, np.float64) - np.asarray(eye, np.float64)
    d /= np.linalg.norm(d)
    return (0.0, 0.0, 1.0) if abs(d[1]) > 0.999 else (0.0, 1.0, 0.0)


def camera_bytes(cam: abi.Camera) -> np.ndarray:
    return np.frombuffer(C.string_at(C.addressof(cam), C.sizeof(cam)), np.uint8).copy()


def grid_camera(width: int = 1920, height: int = 1080, fovy_deg: float = 75.0, moved: float = 0.0) -> abi.Camera:
    """Camera inside the torus grid looking down its long (+x) axis.  With
    `moved`, the previous frame's camera stood that far behind (-x)."""
    gx, gz, gy = GRID
    eye = (0.5 * SPACING * 0.5, (gy / 2 - 0.5) * SPACING, (gz / 2 - 0.5) * SPACING)
    target = (eye[0] + 10.0, eye[1], eye[2])
    prev = None
    if moved:
        prev = camera((eye[0] - moved, eye[1], eye[2]), (target[0] - moved, target[1], target[2]), (0.0, 1.0, 0.0),
                      fovy_deg, width / height)
    return camera(eye, target, (0.0, 1.0, 0.0), fovy_deg, width / height, prev=prev)


BATCH_SIZES = [(256, 256), (512, 384), (1024, 576), (1280, 720), (1920, 1080)]


def batch_views(n: int = 256, radius: float = 30.0, seed: int = 3, fovy_deg: float = 75.0):
    """n seeded eye points uniform on a sphere around the grid centre, aimed
    at it, each with a resolution drawn from BATCH_SIZES."""
    rng = np.random.default_rng(seed)
    centre = grid_centre()
    out = []
    for _ in range(n):
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        eye = centre + radius * v
        w, h = BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))]
        cam = camera(tuple(eye), tuple(centre), safe_up(eye, centre), fovy_deg, w / h)
        out.append((cam, w, h))
    return out
