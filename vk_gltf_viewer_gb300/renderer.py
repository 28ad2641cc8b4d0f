"""Host mirror of the reference's per-frame operator interface over the C ABI.

`Renderer` plays the role of Application's frame recording
(src/vk_gltf_viewer/application.cpp:764-1003): it owns a vkgv context and
issues the culling, visibility-buffer, resolve and HiZ passes for one or many
views.  PyTorch is used only to allocate device memory and to name the CUDA
stream; every pass runs in libvkgv's own sm_103a kernels.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import abi
from .scene import HostScene


def _to_device(arr: np.ndarray, device) -> torch.Tensor:
    raw = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
    if raw.size == 0:
        raw = np.zeros(16, np.uint8)
    return torch.from_numpy(raw.copy()).to(device)


def _ptr(t: torch.Tensor | None) -> int:
    return 0 if t is None else int(t.data_ptr())


def _stream_handle(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


class DeviceScene:
    """Device copies of a HostScene; `.scene` is the vkgv_scene struct."""

    def __init__(self, host: HostScene, device="cuda"):
        self.host = host
        self.device = torch.device(device)
        self._keep = []
        prims = (abi.Primitive * len(host.meshes))()
        for p, mesh in enumerate(host.meshes):
            vi = _to_device(mesh.vertex_indices, self.device)
            pi = _to_device(mesh.primitive_indices, self.device)
            vx = _to_device(mesh.vertices, self.device)
            ml = _to_device(mesh.meshlets, self.device)
            self._keep += [vi, pi, vx, ml]
            prims[p].vertex_index_buffer = _ptr(vi)
            prims[p].primitive_index_buffer = _ptr(pi)
            prims[p].vertex_buffer = _ptr(vx)
            prims[p].meshlet_buffer = _ptr(ml)
            prims[p].aabb_extents[:] = [float(x) for x in mesh.aabb_extents]
            prims[p].aabb_center[:] = [float(x) for x in mesh.aabb_center]
            prims[p].meshlet_count = mesh.meshlet_count
            prims[p].material_index = host.prim_materials[p]
        self.primitives = _to_device(np.frombuffer(bytes(prims), np.uint8), self.device)
        self.draws = _to_device(host.draws.astype(np.uint32), self.device)
        self.transforms = _to_device(host.transforms.astype(np.float32), self.device)
        self.materials = _to_device(host.materials, self.device)
        self.texture_data = [_to_device(t.data, self.device) for t in host.textures]
        table = (abi.Texture * max(1, len(host.textures)))()
        for i, t in enumerate(host.textures):
            table[i].data = _ptr(self.texture_data[i])
            table[i].width = t.width
            table[i].height = t.height
            table[i].format = t.format
            table[i].row_pitch = t.width
        self.texture_table = _to_device(np.frombuffer(bytes(table), np.uint8), self.device)
        # meshlet normal cones (for VKGV_CULL_CONE): one device array per
        # primitive, addressed through a table of device addresses
        self.cone_data = [_to_device(m.cones, self.device) if m.cones is not None and m.cones.size else None
                          for m in host.meshes]
        cone_ptrs = np.array([_ptr(t) for t in self.cone_data], dtype=np.uint64)
        self.cone_table = _to_device(cone_ptrs, self.device)
        self.scene = abi.Scene(draw_buffer=_ptr(self.draws), transform_buffer=_ptr(self.transforms),
                               primitive_buffer=_ptr(self.primitives), material_buffer=_ptr(self.materials),
                               texture_table=_ptr(self.texture_table) if host.textures else 0,
                               meshlet_draw_count=host.draw_count, texture_count=len(host.textures),
                               cone_table=_ptr(self.cone_table), primitive_count=len(host.meshes),
                               transform_count=int(host.transforms.shape[0]))

    @property
    def draw_count(self) -> int:
        return self.host.draw_count


def pyramid_layout(w: int, h: int) -> tuple[int, int]:
    levels, floats = C.c_uint32(), C.c_uint64()
    abi.check(abi.load().vkgv_pyramid_layout(w, h, C.byref(levels), C.byref(floats)))
    return int(levels.value), int(floats.value)


@dataclass
class ViewBuffers:
    """Per-view device images: camera, depth|id, visbuffer, colour, pyramids,
    survivor list and, optionally, the motion-vector image (two binary16 per
    pixel, x in the low half)."""
    width: int
    height: int
    camera: torch.Tensor
    depth_id: torch.Tensor
    visbuffer: torch.Tensor | None
    color: torch.Tensor | None
    pyramid: torch.Tensor | None
    prev_pyramid: torch.Tensor | None
    survivors: torch.Tensor | None
    survivor_count: torch.Tensor | None
    levels: int
    use_prev: bool = True
    motion: torch.Tensor | None = None

    @classmethod
    def allocate(cls, width: int, height: int, cam: abi.Camera, draw_capacity: int, device="cuda",
                 ids: bool = True, color: bool = True, pyramid: bool = True, prev_pyramid: bool = False,
                 survivors: bool = True, motion: bool = False) -> "ViewBuffers":
        dev = torch.device(device)
        levels, floats = pyramid_layout(width, height)
        cam_t = torch.from_numpy(np.frombuffer(C.string_at(C.addressof(cam), C.sizeof(cam)), np.uint8).copy()).to(dev)
        pyr = torch.zeros(max(1, floats), dtype=torch.float32, device=dev) if pyramid and levels else None
        if prev_pyramid == "alias":
            # temporal HiZ in place: the frame reads last frame's pyramid
            # before its own reduce chain overwrites it
            prev = pyr
        else:
            prev = torch.zeros(max(1, floats), dtype=torch.float32, device=dev) if prev_pyramid and levels else None
        return cls(width=width, height=height, camera=cam_t,
                   depth_id=torch.zeros(width * height, dtype=torch.int64, device=dev),
                   visbuffer=torch.zeros(width * height, dtype=torch.int32, device=dev) if ids else None,
                   color=torch.zeros(width * height, dtype=torch.int32, device=dev) if color else None,
                   pyramid=pyr, prev_pyramid=prev,
                   survivors=torch.zeros(max(1, draw_capacity), dtype=torch.int32, device=dev) if survivors else None,
                   survivor_count=torch.zeros(1, dtype=torch.int32, device=dev) if survivors else None,
                   levels=levels,
                   motion=torch.zeros(width * height, dtype=torch.int32, device=dev) if motion else None)

    def set_camera(self, cam: abi.Camera) -> None:
        src = torch.from_numpy(np.frombuffer(C.string_at(C.addressof(cam), C.sizeof(cam)), np.uint8).copy())
        self.camera.copy_(src)

    def struct(self, draw_capacity: int) -> abi.View:
        v = abi.View()
        v.camera_buffer = _ptr(self.camera)
        v.width, v.height = self.width, self.height
        if self.prev_pyramid is not None and self.use_prev:
            v.prev_pyramid = abi.Pyramid(_ptr(self.prev_pyramid), self.width >> 1, self.height >> 1, self.levels, 0)
        if self.pyramid is not None:
            v.pyramid = abi.Pyramid(_ptr(self.pyramid), self.width >> 1, self.height >> 1, self.levels, 0)
        v.depth_id = _ptr(self.depth_id)
        v.visbuffer = _ptr(self.visbuffer)
        v.color = _ptr(self.color)
        v.motion = _ptr(self.motion)
        v.survivors = _ptr(self.survivors)
        v.survivor_count = _ptr(self.survivor_count)
        v.survivor_capacity = 0 if self.survivors is None else int(self.survivors.numel())
        return v

    def motion_vectors(self) -> np.ndarray:
        """The motion image as float32 (H, W, 2)."""
        mv = self.motion.cpu().numpy().view(np.float16).astype(np.float32)
        return mv.reshape(self.height, self.width, 2)

    def survivor_list(self) -> np.ndarray:
        n = int(self.survivor_count.item())
        return self.survivors[:n].cpu().numpy().view(np.uint32).copy()


class Graph:
    def __init__(self, renderer: "Renderer", handle: int, keep):
        self.renderer = renderer
        self.handle = C.c_void_p(handle)
        self._keep = keep

    def launch(self, stream=None) -> None:
        abi.check(abi.load().vkgv_graph_launch(self.handle, _stream_handle(stream)), self.renderer.ctx)

    def kernel_count(self) -> int:
        n = C.c_uint32()
        abi.check(abi.load().vkgv_graph_kernel_count(self.handle, C.byref(n)), self.renderer.ctx)
        return int(n.value)

    def close(self) -> None:
        if self.handle:
            abi.load().vkgv_graph_destroy(self.handle)
            self.handle = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Renderer:
    """Owns one vkgv context on one CUDA device."""

    def __init__(self, device: int = 0, bin_size: int = 0, meshlets_per_cta: int = 0, big_capacity: int = 0):
        if not torch.cuda.is_available():
            raise RuntimeError("vkgv Renderer needs a CUDA device")
        self.lib = abi.load()
        torch.cuda.set_device(device)
        torch.cuda.init()
        cfg = abi.Config(device=device, bin_size=bin_size, meshlets_per_cta=meshlets_per_cta,
                         big_triangle_capacity=big_capacity)
        ctx = C.c_void_p()
        abi.check(self.lib.vkgv_create(C.byref(cfg), C.byref(ctx)))
        self.ctx = ctx
        self.device = device
        self.bin_size = bin_size
        self.meshlets_per_cta = meshlets_per_cta
        self.big_capacity = big_capacity

    def close(self) -> None:
        if self.ctx:
            self.lib.vkgv_destroy(self.ctx)
            self.ctx = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _views(self, scene: DeviceScene, views: list[ViewBuffers]):
        arr = (abi.View * len(views))()
        for i, v in enumerate(views):
            arr[i] = v.struct(scene.draw_count)
        return arr

    def frame(self, scene: DeviceScene, views: list[ViewBuffers], flags: int = abi.FRAME_REFERENCE,
              stream=None) -> None:
        arr = self._views(scene, views)
        abi.check(self.lib.vkgv_frame(self.ctx, C.byref(scene.scene), arr, len(views), flags,
                                      _stream_handle(stream)), self.ctx)

    def clear(self, scene: DeviceScene, view: ViewBuffers, stream=None) -> None:
        v = view.struct(scene.draw_count)
        abi.check(self.lib.vkgv_clear(self.ctx, C.byref(v), _stream_handle(stream)), self.ctx)

    def cull(self, scene: DeviceScene, view: ViewBuffers, flags: int, pass_: int = 1, stream=None) -> None:
        v = view.struct(scene.draw_count)
        abi.check(self.lib.vkgv_cull(self.ctx, C.byref(scene.scene), C.byref(v), flags, pass_,
                                     _stream_handle(stream)), self.ctx)

    def raster(self, scene: DeviceScene, view: ViewBuffers, draw_list: torch.Tensor | None = None,
               draw_count: torch.Tensor | None = None, first: int = 0, stream=None) -> None:
        v = view.struct(scene.draw_count)
        abi.check(self.lib.vkgv_raster(self.ctx, C.byref(scene.scene), C.byref(v), _ptr(draw_list),
                                       _ptr(draw_count), first, _stream_handle(stream)), self.ctx)

    def hiz(self, scene: DeviceScene, view: ViewBuffers, stream=None) -> None:
        v = view.struct(scene.draw_count)
        abi.check(self.lib.vkgv_hiz_reduce(self.ctx, C.byref(v), _stream_handle(stream)), self.ctx)

    def resolve(self, scene: DeviceScene, view: ViewBuffers, flags: int = abi.RESOLVE_FLAT | abi.WRITE_IDS,
                stream=None) -> None:
        v = view.struct(scene.draw_count)
        abi.check(self.lib.vkgv_resolve(self.ctx, C.byref(scene.scene), C.byref(v), flags,
                                        _stream_handle(stream)), self.ctx)

    def capture(self, scene: DeviceScene, views: list[ViewBuffers], flags: int = abi.FRAME_REFERENCE) -> Graph:
        arr = self._views(scene, views)
        g = C.c_void_p()
        abi.check(self.lib.vkgv_graph_capture(self.ctx, C.byref(scene.scene), arr, len(views), flags, C.byref(g)),
                  self.ctx)
        return Graph(self, g.value, (scene, views))

    def sweep(self, scene: DeviceScene, views: list[ViewBuffers], flags: int, launches: int = 3):
        """Native launch-shape sweep (vkgv_autotune) over this workload.
        Returns ([(bin_size, meshlets_per_cta, ms_per_launch)], best (bin, split))."""
        arr = self._views(scene, views)
        base = abi.Config(device=self.device, big_triangle_capacity=self.big_capacity)
        entries = (abi.TuneEntry * 16)()
        n = C.c_uint32()
        best = abi.Config()
        abi.check(self.lib.vkgv_autotune(C.byref(base), C.byref(scene.scene), arr, len(views), flags, launches,
                                         entries, 16, C.byref(n), C.byref(best)))
        table = [(int(e.bin_size), int(e.meshlets_per_cta), float(e.ms_per_launch)) for e in entries[:n.value]]
        return table, (int(best.bin_size), int(best.meshlets_per_cta))

    def set_profiling(self, enable: bool) -> None:
        abi.check(self.lib.vkgv_set_profiling(self.ctx, 1 if enable else 0), self.ctx)

    def stage_times(self) -> dict[str, float]:
        """Milliseconds per stage of the last profiled vkgv_frame."""
        out = (C.c_float * abi.STAGE_COUNT)()
        abi.check(self.lib.vkgv_stage_times(self.ctx, out, abi.STAGE_COUNT), self.ctx)
        return dict(zip(abi.STAGE_NAMES, [float(x) for x in out]))

    def device_status(self) -> tuple[int, int]:
        code, detail = C.c_uint32(), C.c_uint32()
        abi.check(self.lib.vkgv_device_status(self.ctx, C.byref(code), C.byref(detail)), self.ctx)
        return int(code.value), int(detail.value)
