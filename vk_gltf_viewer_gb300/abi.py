"""ctypes mirror of include/vkgv.h and the loader of libvkgv.so.

The library is loaded from the package directory only (an in-tree build).
Loading fails loudly when it is missing: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
HEADER = ROOT / "include" / "vkgv.h"
LIB_PATH = PKG / "libvkgv.so"

# status codes
OK, INVALID_ARG, OUT_OF_MEMORY, LIMIT_EXCEEDED, TIMEOUT, CUDA_ERROR, DEVICE_FAULT = range(7)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "LIMIT_EXCEEDED", 4: "TIMEOUT",
                5: "CUDA_ERROR", 6: "DEVICE_FAULT"}

MAX_VERTICES = 64
MAX_PRIMITIVES = 126
MAX_MESHLETS = 102
BUILDER_MAX_TRIANGLES = 124
TRIANGLE_BITS = 7
DRAW_INDEX_BITS = 25
VISBUFFER_CLEAR = 0xFFFFFFFF
INVALID_HANDLE = 0xFFFFFFFF
MAX_VIEW_DIM = 8192

# frame flags
CULL_FRUSTUM = 1 << 0
CULL_OCCLUSION = 1 << 1
CULL_TWO_PASS = 1 << 2
CULL_CONE = 1 << 3
RESOLVE_FLAT = 1 << 4
RESOLVE_TEXTURED = 1 << 5
BUILD_PYRAMID = 1 << 6
WRITE_IDS = 1 << 7
SKIP_CLEAR = 1 << 8
WRITE_MOTION = 1 << 9
CULL_OCCLUSION_FINE = 1 << 10

# passes of vkgv_diff_graph_capture
DIFF_ZERO_GRADS = 1
DIFF_FORWARD = 2
DIFF_BACKWARD = 4
FRAME_REFERENCE = CULL_FRUSTUM | CULL_OCCLUSION | RESOLVE_FLAT | BUILD_PYRAMID | WRITE_IDS

STAGE_COUNT = 11
STAGE_NAMES = ["clear", "cull1", "raster1", "big1", "hiz1", "cull2", "raster2", "big2", "hiz",
               "resolve", "finalize"]

TEXTURE_RGBA8 = 0
TEXTURE_RGB32F = 1


class Meshlet(C.Structure):
    _fields_ = [("vertex_offset", C.c_uint32), ("triangle_offset", C.c_uint32),
                ("vertex_count", C.c_uint8), ("triangle_count", C.c_uint8), ("_pad", C.c_uint8 * 2),
                ("aabb_extents", C.c_float * 3), ("aabb_center", C.c_float * 3)]


class Vertex(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_uint8 * 4), ("normal", C.c_uint8 * 3),
                ("_pad", C.c_uint8), ("uv", C.c_uint16 * 2)]


class MeshletDraw(C.Structure):
    _fields_ = [("primitive_index", C.c_uint32), ("meshlet_index", C.c_uint32), ("transform_index", C.c_uint32)]


class Primitive(C.Structure):
    _fields_ = [("vertex_index_buffer", C.c_uint64), ("primitive_index_buffer", C.c_uint64),
                ("vertex_buffer", C.c_uint64), ("meshlet_buffer", C.c_uint64),
                ("aabb_extents", C.c_float * 3), ("aabb_center", C.c_float * 3),
                ("meshlet_count", C.c_uint32), ("material_index", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("albedo_factor", C.c_float * 4), ("albedo_index", C.c_uint32), ("uv_offset", C.c_float * 2),
                ("uv_scale", C.c_float * 2), ("uv_rotation", C.c_float), ("alpha_cutoff", C.c_float),
                ("double_sided", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("prev_view_projection", C.c_float * 16), ("prev_occlusion_view_projection", C.c_float * 16),
                ("view_projection", C.c_float * 16), ("occlusion_view_projection", C.c_float * 16),
                ("frustum", C.c_float * 24)]


class Texture(C.Structure):
    _fields_ = [("data", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32),
                ("row_pitch", C.c_uint32)]


class Pyramid(C.Structure):
    _fields_ = [("data", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32), ("levels", C.c_uint32),
                ("_pad", C.c_uint32)]


class Scene(C.Structure):
    _fields_ = [("draw_buffer", C.c_uint64), ("transform_buffer", C.c_uint64), ("primitive_buffer", C.c_uint64),
                ("material_buffer", C.c_uint64), ("texture_table", C.c_uint64),
                ("meshlet_draw_count", C.c_uint32), ("texture_count", C.c_uint32),
                ("cone_table", C.c_uint64), ("primitive_count", C.c_uint32), ("transform_count", C.c_uint32)]


class MeshletCone(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("axis", C.c_float * 3), ("cutoff", C.c_float)]


class View(C.Structure):
    _fields_ = [("camera_buffer", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("prev_pyramid", Pyramid), ("pyramid", Pyramid), ("depth_id", C.c_uint64),
                ("visbuffer", C.c_uint64), ("color", C.c_uint64), ("survivors", C.c_uint64),
                ("survivor_count", C.c_uint64), ("survivor_capacity", C.c_uint32), ("_pad", C.c_uint32),
                ("motion", C.c_uint64)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("bin_size", C.c_uint32), ("meshlets_per_cta", C.c_uint32),
                ("big_triangle_capacity", C.c_uint32), ("spin_limit", C.c_uint32), ("_reserved", C.c_uint32 * 3)]


class TuneEntry(C.Structure):
    _fields_ = [("bin_size", C.c_uint32), ("meshlets_per_cta", C.c_uint32), ("ms_per_launch", C.c_float),
                ("_pad", C.c_uint32)]


class MeshInfo(C.Structure):
    _fields_ = [("vertex_count", C.c_uint32), ("triangle_count", C.c_uint32), ("meshlet_count", C.c_uint32),
                ("vertex_index_count", C.c_uint32), ("primitive_index_bytes", C.c_uint32),
                ("position_scale", C.c_float),
                ("vertices", C.POINTER(Vertex)), ("positions", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
                ("indices", C.POINTER(C.c_uint32)), ("meshlets", C.POINTER(Meshlet)),
                ("vertex_indices", C.POINTER(C.c_uint32)), ("primitive_indices", C.POINTER(C.c_uint8)),
                ("aabb_extents", C.c_float * 3), ("aabb_center", C.c_float * 3),
                ("cones", C.POINTER(MeshletCone))]


class DiffScene(C.Structure):
    _fields_ = [("meshlet_buffer", C.c_uint64), ("vertex_index_buffer", C.c_uint64),
                ("primitive_index_buffer", C.c_uint64), ("positions", C.c_uint64), ("colors", C.c_uint64),
                ("uvs", C.c_uint64), ("texture", C.c_uint64), ("meshlet_count", C.c_uint32),
                ("vertex_count", C.c_uint32), ("tex_width", C.c_uint32), ("tex_height", C.c_uint32),
                ("albedo", C.c_float * 3), ("uv_offset", C.c_float * 2), ("uv_scale", C.c_float * 2),
                ("uv_rotation", C.c_float), ("double_sided", C.c_uint32), ("cone_mode", C.c_uint32)]


class DiffView(C.Structure):
    _fields_ = [("camera_buffer", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("depth_id", C.c_uint64), ("rgb", C.c_uint64), ("target", C.c_uint64), ("grad_rgb", C.c_uint64)]


class Node(C.Structure):
    _fields_ = [("translation", C.c_float * 3), ("rotation", C.c_float * 4), ("scale", C.c_float * 3),
                ("mesh_index", C.c_uint32), ("first_child", C.c_uint32), ("child_count", C.c_uint32)]


class AnimSampler(C.Structure):
    _fields_ = [("input", C.c_void_p), ("output", C.c_void_p), ("input_count", C.c_uint32),
                ("output_count", C.c_uint32), ("interpolation", C.c_uint32), ("components", C.c_uint32)]


class AnimChannel(C.Structure):
    _fields_ = [("sampler", C.c_uint32), ("node", C.c_uint32), ("path", C.c_uint32), ("_pad", C.c_uint32)]


class WorldDesc(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("node_count", C.c_uint32), ("child_count", C.c_uint32),
                ("children", C.c_void_p), ("roots", C.c_void_p), ("root_count", C.c_uint32),
                ("mesh_count", C.c_uint32), ("mesh_offsets", C.c_void_p), ("mesh_primitives", C.c_void_p),
                ("primitive_meshlet_counts", C.c_void_p), ("primitive_count", C.c_uint32),
                ("sampler_count", C.c_uint32), ("samplers", C.c_void_p), ("channels", C.c_void_p),
                ("channel_count", C.c_uint32), ("_pad", C.c_uint32)]


class GltfInfo(C.Structure):
    _fields_ = [("primitive_count", C.c_uint32), ("material_count", C.c_uint32), ("mesh_count", C.c_uint32),
                ("node_count", C.c_uint32), ("root_count", C.c_uint32), ("sampler_count", C.c_uint32),
                ("channel_count", C.c_uint32), ("texture_count", C.c_uint32), ("image_count", C.c_uint32),
                ("_pad", C.c_uint32)]


class GltfPrimitive(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("material_index", C.c_uint32), ("mesh_index", C.c_uint32),
                ("meshlet_count", C.c_uint32), ("_pad", C.c_uint32)]


class GltfImage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("size", C.c_uint64), ("kind", C.c_uint32), ("_pad", C.c_uint32)]


class DdsInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("mip_count", C.c_uint32), ("format", C.c_uint32),
                ("srgb", C.c_uint32), ("supercompression", C.c_uint32), ("data_offset", C.c_uint64),
                ("data_size", C.c_uint64)]


class JpegInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("components", C.c_uint32), ("rgb", C.c_uint32),
                ("hmax", C.c_uint32), ("vmax", C.c_uint32), ("h", C.c_uint32 * 3), ("v", C.c_uint32 * 3),
                ("blocks_w", C.c_uint32 * 3), ("blocks_h", C.c_uint32 * 3)]


GLTF_TEXTURE_REFERENCES = 1
GLTF_IMAGES = 2
IMAGE_UNKNOWN, IMAGE_PNG, IMAGE_DDS, IMAGE_JPEG, IMAGE_KTX2 = 0, 1, 2, 3, 4
BC1, BC2, BC3, BC4, BC5, BC1_OPAQUE, RGBA8, BC7, BC6H_UF16, BC6H_SF16 = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
BGRA8, RGBX8, BGRX8 = 11, 12, 13  # uncompressed DDS texels (host)
PATH_TRANSLATION, PATH_ROTATION, PATH_SCALE, PATH_WEIGHTS = 1, 2, 3, 4
INTERP_LINEAR, INTERP_STEP, INTERP_CUBICSPLINE = 0, 1, 2
MAX_NODE_DEPTH = 64
MESHOPT_ATTRIBUTES, MESHOPT_TRIANGLES, MESHOPT_INDICES = 0, 1, 2
MESHOPT_FILTER_NONE, MESHOPT_FILTER_OCTAHEDRAL, MESHOPT_FILTER_QUATERNION, MESHOPT_FILTER_EXPONENTIAL = 0, 1, 2, 3

EXPECTED_SIZES = {"Meshlet": 36, "Vertex": 24, "MeshletDraw": 12, "Primitive": 64, "Material": 48, "Camera": 352,
                  "Node": 52, "AnimSampler": 32, "AnimChannel": 16, "WorldDesc": 96,
                  "GltfInfo": 40, "GltfPrimitive": 24, "GltfImage": 24, "DdsInfo": 40, "JpegInfo": 72}

_P = C.c_void_p
_U32 = C.c_uint32
_U64 = C.c_uint64
_PROTOS = {
    "vkgv_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "vkgv_destroy": (C.c_int, [_P]),
    "vkgv_last_error": (C.c_char_p, [_P]),
    "vkgv_device_status": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U32)]),
    "vkgv_frame": (C.c_int, [_P, C.POINTER(Scene), C.POINTER(View), _U32, _U32, _P]),
    "vkgv_clear": (C.c_int, [_P, C.POINTER(View), _P]),
    "vkgv_cull": (C.c_int, [_P, C.POINTER(Scene), C.POINTER(View), _U32, _U32, _P]),
    "vkgv_cull_static": (C.c_int, [C.POINTER(Scene), C.POINTER(View), _U32, _U32, _P]),
    "vkgv_cull_static_status": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U32)]),
    "vkgv_zstd_decompress": (C.c_int, [_P, _U64, _P, _U64, C.POINTER(_U64)]),
    "vkgv_xxh64": (_U64, [_P, _U64]),
    "vkgv_raster": (C.c_int, [_P, C.POINTER(Scene), C.POINTER(View), _U64, _U64, _U32, _P]),
    "vkgv_hiz_reduce": (C.c_int, [_P, C.POINTER(View), _P]),
    "vkgv_resolve": (C.c_int, [_P, C.POINTER(Scene), C.POINTER(View), _U32, _P]),
    "vkgv_pyramid_layout": (C.c_int, [_U32, _U32, C.POINTER(_U32), C.POINTER(_U64)]),
    "vkgv_graph_capture": (C.c_int, [_P, C.POINTER(Scene), C.POINTER(View), _U32, _U32, C.POINTER(_P)]),
    "vkgv_graph_launch": (C.c_int, [_P, _P]),
    "vkgv_graph_destroy": (C.c_int, [_P]),
    "vkgv_graph_kernel_count": (C.c_int, [_P, C.POINTER(_U32)]),
    "vkgv_mesh_icosphere": (_P, [_U32]),
    "vkgv_mesh_torus": (_P, [C.c_float, C.c_float, _U32, _U32, C.c_float, _U64, C.c_int32]),
    "vkgv_mesh_displace": (C.c_int, [_P, C.c_float, _U64]),
    "vkgv_mesh_from_arrays": (_P, [C.POINTER(C.c_float), _U32, C.POINTER(_U32), _U32]),
    "vkgv_mesh_set_attributes": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "vkgv_mesh_build_meshlets": (C.c_int, [_P, _U32, _U32]),
    "vkgv_mesh_get_info": (C.c_int, [_P, C.POINTER(MeshInfo)]),
    "vkgv_mesh_free": (None, [_P]),
    "vkgv_camera_update": (C.c_int, [C.POINTER(Camera), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float, C.c_float]),
    "vkgv_frustum_planes": (C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "vkgv_version": (C.c_char_p, []),
    "vkgv_diff_forward": (C.c_int, [_P, C.POINTER(DiffScene), C.POINTER(DiffView), _U32, _P]),
    "vkgv_diff_backward": (C.c_int, [_P, C.POINTER(DiffScene), C.POINTER(DiffView), _U32, C.c_float, _U64, _U64,
                                     _U64, _U64, _P]),
    "vkgv_diff_graph_capture": (C.c_int, [_P, C.POINTER(DiffScene), C.POINTER(DiffView), _U32, _U32, C.c_float,
                                          _U64, _U64, _U64, _U64, C.POINTER(_P)]),
    "vkgv_autotune": (C.c_int, [C.POINTER(Config), C.POINTER(Scene), C.POINTER(View), _U32, _U32, _U32,
                                C.POINTER(TuneEntry), _U32, C.POINTER(_U32), C.POINTER(Config)]),
    "vkgv_world_create": (C.c_int, [_P, C.POINTER(WorldDesc), C.POINTER(_P)]),
    "vkgv_world_destroy": (C.c_int, [_P]),
    "vkgv_world_info": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U64)]),
    "vkgv_world_update_transforms": (C.c_int, [_P, _P, C.c_float, _U64, _P]),
    "vkgv_world_build_draws": (C.c_int, [_P, _P, _U64, _U64, _P]),
    "vkgv_gltf_load": (C.c_int, [C.c_char_p, _U32, C.POINTER(_P), C.c_char_p, _U32]),
    "vkgv_gltf_get_info": (C.c_int, [_P, C.POINTER(GltfInfo)]),
    "vkgv_gltf_get_primitive": (C.c_int, [_P, _U32, C.POINTER(GltfPrimitive)]),
    "vkgv_gltf_get_materials": (C.c_int, [_P, _P, _U32]),
    "vkgv_gltf_get_world": (C.c_int, [_P, C.POINTER(WorldDesc)]),
    "vkgv_gltf_get_texture_image": (C.c_int, [_P, _U32, C.POINTER(GltfImage)]),
    "vkgv_gltf_free": (None, [_P]),
    "vkgv_meshopt_decode": (C.c_int, [_P, _U64, _U64, _P, _U64, C.c_int, C.c_int]),
    "vkgv_image_decode_png": (C.c_int, [_P, _U64, C.POINTER(_P), C.c_char_p, _U32]),
    "vkgv_image_get": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(_P)]),
    "vkgv_image_free": (None, [_P]),
    "vkgv_dds_parse": (C.c_int, [_P, _U64, C.POINTER(DdsInfo)]),
    "vkgv_ktx2_parse": (C.c_int, [_P, _U64, C.POINTER(DdsInfo)]),
    "vkgv_decode_bc": (C.c_int, [_P, _U32, _U64, _U32, _U32, _U64, _P]),
    "vkgv_decode_bc6h": (C.c_int, [_P, _U32, _U64, _U32, _U32, _U64, _P]),
    "vkgv_jpeg_decode_coefficients": (C.c_int, [_P, _U64, C.POINTER(_P), C.c_char_p, _U32]),
    "vkgv_jpeg_get_info": (C.c_int, [_P, C.POINTER(JpegInfo)]),
    "vkgv_jpeg_get_coefficients": (C.c_int, [_P, _U32, C.POINTER(_P)]),
    "vkgv_jpeg_to_rgba": (C.c_int, [_P, _P, _U64, _P]),
    "vkgv_jpeg_free": (None, [_P]),
    "vkgv_set_profiling": (C.c_int, [_P, C.c_int32]),
    "vkgv_stage_times": (C.c_int, [_P, C.POINTER(C.c_float), _U32]),
}

_lib = None


class VkgvError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


def declared_symbols() -> list[str]:
    """Function names declared in include/vkgv.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vkgv_[a-z0-9_]+)\s*\(", text)))


def load() -> C.CDLL:
    """Loads the in-tree libvkgv.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | os.RTLD_LOCAL)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, ctx=None) -> None:
    if code != OK:
        msg = ""
        if ctx is not None:
            raw = load().vkgv_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise VkgvError(code, msg)
