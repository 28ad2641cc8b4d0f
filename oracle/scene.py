"""Scene and camera producers of the oracle (oracle/scene.c through ctypes,
the scene assembly in numpy).  TEST INFRASTRUCTURE ONLY: the benchmark's
reference arm builds its C1/C2 inputs here so that it never loads the product
library, and a CPU test checks every buffer against the product's producers
byte for byte.

The assembly follows the reference's draw-list order, node -> primitive ->
meshlet (src/vk_gltf_viewer/world.cpp:245-262), material 0 as the glTF default
with glTF material i stored at i + 1 (src/vk_gltf_viewer/assets.cpp:292-294,
486-492), and the camera update of src/vk_gltf_viewer/camera.cpp:170-193.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import binding

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
INVALID_HANDLE = 0xFFFFFFFF
TEXTURE_RGBA8 = 0

GRID = (16, 16, 8)   # x, z (long axes) and y (layers)
SPACING = 2.5
BATCH_SIZES = [(256, 256), (512, 384), (1024, 576), (1280, 720), (1920, 1080)]


class Camera(C.Structure):
    """The 352-byte camera buffer (shaders/mesh_common.h.glsl:20-27)."""
    _fields_ = [("prev_view_projection", C.c_float * 16), ("prev_occlusion_view_projection", C.c_float * 16),
                ("view_projection", C.c_float * 16), ("occlusion_view_projection", C.c_float * 16),
                ("frustum", C.c_float * 24)]


class _MeshInfo(C.Structure):
    _fields_ = [("vertex_count", C.c_uint32), ("triangle_count", C.c_uint32), ("meshlet_count", C.c_uint32),
                ("vertex_index_count", C.c_uint32), ("primitive_index_bytes", C.c_uint32),
                ("position_scale", C.c_float), ("vertices", C.c_void_p), ("positions", C.c_void_p),
                ("uvs", C.c_void_p), ("indices", C.c_void_p), ("meshlets", C.c_void_p),
                ("vertex_indices", C.c_void_p), ("primitive_indices", C.c_void_p), ("cones", C.c_void_p),
                ("aabb_extents", C.c_float * 3), ("aabb_center", C.c_float * 3)]


_bound = False


def _lib():
    global _bound
    lib = binding.load()
    if not _bound:
        P = C.c_void_p
        lib.orc_mesh_icosphere.restype = P
        lib.orc_mesh_icosphere.argtypes = [C.c_uint32]
        lib.orc_mesh_torus.restype = P
        lib.orc_mesh_torus.argtypes = [C.c_float, C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64,
                                       C.c_int32]
        lib.orc_mesh_displace.argtypes = [P, C.c_float, C.c_uint64]
        lib.orc_mesh_build_meshlets.argtypes = [P, C.c_uint32, C.c_uint32]
        lib.orc_mesh_get_info.argtypes = [P, P]
        lib.orc_mesh_free.argtypes = [P]
        lib.orc_camera_update.argtypes = [P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float]
        _bound = True
    return lib


@dataclass
class Mesh:
    vertices: np.ndarray
    positions: np.ndarray
    uvs: np.ndarray | None
    indices: np.ndarray
    meshlets: np.ndarray
    vertex_indices: np.ndarray
    primitive_indices: np.ndarray
    aabb_extents: np.ndarray
    aabb_center: np.ndarray
    position_scale: float = 1.0
    cones: np.ndarray | None = None

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
    return np.frombuffer(C.string_at(ptr, n * dtype.itemsize), dtype=dtype, count=n).copy()


def _take(h, max_vertices: int = 64, max_triangles: int = 124) -> Mesh:
    lib = _lib()
    if not h:
        raise ValueError("oracle mesh producer failed")
    try:
        if lib.orc_mesh_build_meshlets(h, max_vertices, max_triangles) != 0:
            raise ValueError("oracle meshletiser failed")
        info = _MeshInfo()
        lib.orc_mesh_get_info(h, C.byref(info))
        nv, nt = info.vertex_count, info.triangle_count
        return Mesh(vertices=_copy(info.vertices, nv, VERTEX_DTYPE),
                    positions=_copy(info.positions, nv * 3, np.float32).reshape(nv, 3),
                    uvs=_copy(info.uvs, nv * 2, np.float32).reshape(nv, 2) if info.uvs else None,
                    indices=_copy(info.indices, nt * 3, np.uint32).reshape(nt, 3),
                    meshlets=_copy(info.meshlets, info.meshlet_count, MESHLET_DTYPE),
                    vertex_indices=_copy(info.vertex_indices, info.vertex_index_count, np.uint32),
                    primitive_indices=_copy(info.primitive_indices, info.primitive_index_bytes, np.uint8),
                    aabb_extents=np.array(info.aabb_extents[:], np.float32),
                    aabb_center=np.array(info.aabb_center[:], np.float32),
                    position_scale=float(info.position_scale),
                    cones=_copy(info.cones, info.meshlet_count, CONE_DTYPE))
    finally:
        lib.orc_mesh_free(h)


def icosphere(level: int, displace: float = 0.0, seed: int = 0) -> Mesh:
    lib = _lib()
    h = lib.orc_mesh_icosphere(level)
    if displace:
        lib.orc_mesh_displace(h, displace, seed)
    return _take(h)


def torus(R: float = 1.0, r: float = 0.35, seg_major: int = 200, seg_minor: int = 100, noise_amp: float = 0.05,
          seed: int = 1, quantize: bool = True) -> Mesh:
    return _take(_lib().orc_mesh_torus(R, r, seg_major, seg_minor, noise_amp, seed, 1 if quantize else 0))


@dataclass
class Texture:
    data: np.ndarray
    format: int

    @property
    def width(self) -> int:
        return int(self.data.shape[1])

    @property
    def height(self) -> int:
        return int(self.data.shape[0])


@dataclass
class HostScene:
    meshes: list[Mesh]
    prim_materials: list[int]
    materials: np.ndarray
    transforms: np.ndarray
    node_meshes: list[list[int]]
    textures: list[Texture] = field(default_factory=list)
    draws: np.ndarray | None = None

    def __post_init__(self):
        if self.draws is None:
            parts = []
            for t, prims in enumerate(self.node_meshes):
                for p in prims:
                    n = self.meshes[p].meshlet_count
                    d = np.empty((n, 3), np.uint32)
                    d[:, 0] = p
                    d[:, 1] = np.arange(n, dtype=np.uint32)
                    d[:, 2] = t
                    parts.append(d)
            self.draws = np.ascontiguousarray(np.concatenate(parts)) if parts else np.zeros((0, 3), np.uint32)

    @property
    def draw_count(self) -> int:
        return int(self.draws.shape[0])

    @property
    def triangle_count(self) -> int:
        return int(sum(self.meshes[p].triangle_count for prims in self.node_meshes for p in prims))


def _material(albedo=(1.0, 1.0, 1.0, 1.0), albedo_index=INVALID_HANDLE, uv_scale=(1.0, 1.0)) -> np.ndarray:
    m = np.zeros(1, MATERIAL_DTYPE)
    m["albedo_factor"] = albedo
    m["albedo_index"] = albedo_index
    m["uv_offset"] = (0.0, 0.0)
    m["uv_scale"] = uv_scale
    m["uv_rotation"] = 0.0
    m["alpha_cutoff"] = 0.5
    m["double_sided"] = 0
    return m


def _column_major(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float64).T.reshape(16), np.float32)


def scene_icosphere(level: int = 6, albedo=(0.8, 0.5, 0.3, 1.0)) -> HostScene:
    """One icosphere node, material 1 of constant base colour."""
    mats = np.concatenate([_material(), _material(albedo)])
    return HostScene(meshes=[icosphere(level)], prim_materials=[1], materials=mats,
                     transforms=_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])


def grid_centre() -> np.ndarray:
    gx, gz, gy = GRID
    return np.array([(gx - 1) * SPACING / 2, (gy - 1) * SPACING / 2, (gz - 1) * SPACING / 2])


def scene_torus_grid(seed: int = 7, texture_size: int = 2048, grid=GRID, tex_seed: int = 11) -> HostScene:
    """The displaced, quantised torus instanced on a 16 x 16 x 8 grid
    (spacing 2.5, seeded yaw, the dequantisation scale in each node matrix)
    with one RGBA8 noise texture under a KHR_texture_transform scale of 4."""
    mesh = torus(seed=seed)
    rng = np.random.default_rng(seed)
    gx, gz, gy = grid
    s = mesh.position_scale
    transforms = []
    for k in range(gy):
        for j in range(gz):
            for i in range(gx):
                yaw = rng.uniform(0, 2 * math.pi)
                c, sn = math.cos(yaw), math.sin(yaw)
                t = np.eye(4)
                t[:3, 3] = (i * SPACING, k * SPACING, j * SPACING)
                r = np.eye(4)
                r[0, 0], r[0, 2], r[2, 0], r[2, 2] = c, sn, -sn, c
                sc = np.diag([s, s, s, 1.0])
                transforms.append(_column_major(t @ r @ sc))
    textures = []
    albedo_index = INVALID_HANDLE
    if texture_size:
        trng = np.random.default_rng(tex_seed)
        tex = trng.integers(0, 256, size=(texture_size, texture_size, 4), dtype=np.uint8)
        tex[..., 3] = 255
        textures.append(Texture(tex, TEXTURE_RGBA8))
        albedo_index = 0
    mats = np.concatenate([_material(), _material(albedo_index=albedo_index, uv_scale=(4.0, 4.0))])
    tr = np.stack(transforms)
    return HostScene(meshes=[mesh], prim_materials=[1], materials=mats, transforms=tr,
                     node_meshes=[[0] for _ in range(tr.shape[0])], textures=textures)


def camera(eye, target, up=(0.0, 1.0, 0.0), fovy_deg: float = 60.0, aspect: float = 16 / 9, znear: float = 0.1,
           zfar: float = 1000.0) -> Camera:
    """Camera buffer of a static camera (two updates: prev = current)."""
    cam = Camera()
    e, t, u = (C.c_float * 3)(*eye), (C.c_float * 3)(*target), (C.c_float * 3)(*up)
    for _ in range(2):
        if _lib().orc_camera_update(C.byref(cam), e, t, u, math.radians(fovy_deg), aspect, znear, zfar) != 0:
            raise ValueError("oracle camera update failed")
    return cam


def grid_camera(width: int = 1920, height: int = 1080, fovy_deg: float = 75.0) -> Camera:
    """Inside the torus grid, looking down its long (+x) axis."""
    gx, gz, gy = GRID
    eye = (0.5 * SPACING * 0.5, (gy / 2 - 0.5) * SPACING, (gz / 2 - 0.5) * SPACING)
    return camera(eye, (eye[0] + 10.0, eye[1], eye[2]), (0.0, 1.0, 0.0), fovy_deg, width / height)


def icosphere_camera(width: int = 1280, height: int = 720) -> Camera:
    """Eye (0, 0, 3) looking at the origin, 60 degree vertical field of view."""
    return camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, width / height)


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
        d = centre - eye
        d = d / np.linalg.norm(d)
        up = (0.0, 0.0, 1.0) if abs(d[1]) > 0.999 else (0.0, 1.0, 0.0)
        out.append((camera(tuple(eye), tuple(centre), up, fovy_deg, w / h), w, h))
    return out
