"""Differentiable textured resolve (the adjoint addition) over the C ABI.

A `DiffScene` holds a meshletised mesh and its fp32 parameters (positions,
per-vertex linear RGB colours, UVs and an fp32 RGB texture) as device
tensors.  `forward` renders linear RGB per view; `backward` recomputes the
visibility and accumulates gradients with respect to positions, colours and
texels, given either an MSE target or an upstream dL/drgb.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import abi
from .renderer import Graph, Renderer, _ptr, _stream_handle
from .scene import Mesh


@dataclass
class DiffScene:
    mesh: Mesh
    meshlets: torch.Tensor
    vertex_indices: torch.Tensor
    primitive_indices: torch.Tensor
    positions: torch.Tensor   # (V, 3) float32
    colors: torch.Tensor      # (V, 3) float32
    uvs: torch.Tensor         # (V, 2) float32
    texture: torch.Tensor     # (H, W, 3) float32
    albedo: tuple = (1.0, 1.0, 1.0)
    uv_offset: tuple = (0.0, 0.0)
    uv_scale: tuple = (1.0, 1.0)
    uv_rotation: float = 0.0
    double_sided: bool = False
    cone_mode: int = 0  # meshlet cone culling: 0 automatic, 1 always, 2 never

    @classmethod
    def create(cls, mesh: Mesh, colors: np.ndarray, texture: np.ndarray, device="cuda",
               positions: np.ndarray | None = None, **kw) -> "DiffScene":
        dev = torch.device(device)

        def u8(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).to(dev)

        pos = mesh.positions if positions is None else positions
        return cls(mesh=mesh, meshlets=u8(mesh.meshlets), vertex_indices=u8(mesh.vertex_indices),
                   primitive_indices=u8(mesh.primitive_indices),
                   positions=torch.tensor(np.asarray(pos, np.float32), device=dev).contiguous(),
                   colors=torch.tensor(np.asarray(colors, np.float32), device=dev).contiguous(),
                   uvs=torch.tensor(np.asarray(mesh.uvs, np.float32), device=dev).contiguous(),
                   texture=torch.tensor(np.asarray(texture, np.float32), device=dev).contiguous(), **kw)

    def struct(self, positions=None, colors=None, texture=None) -> abi.DiffScene:
        pos = self.positions if positions is None else positions
        col = self.colors if colors is None else colors
        tex = self.texture if texture is None else texture
        for t in (pos, col, tex):
            if t.dtype != torch.float32 or not t.is_contiguous():
                raise ValueError("adjoint parameters must be contiguous float32 tensors")
        s = abi.DiffScene()
        s.meshlet_buffer = _ptr(self.meshlets)
        s.vertex_index_buffer = _ptr(self.vertex_indices)
        s.primitive_index_buffer = _ptr(self.primitive_indices)
        s.positions, s.colors, s.uvs, s.texture = _ptr(pos), _ptr(col), _ptr(self.uvs), _ptr(tex)
        s.meshlet_count = self.mesh.meshlet_count
        s.vertex_count = int(pos.shape[0])
        s.tex_width, s.tex_height = int(tex.shape[1]), int(tex.shape[0])
        s.albedo[:] = list(self.albedo)
        s.uv_offset[:] = list(self.uv_offset)
        s.uv_scale[:] = list(self.uv_scale)
        s.uv_rotation = float(self.uv_rotation)
        s.double_sided = 1 if self.double_sided else 0
        s.cone_mode = int(self.cone_mode)
        return s


@dataclass
class DiffViewBuffers:
    width: int
    height: int
    camera: torch.Tensor
    depth_id: torch.Tensor

    @classmethod
    def allocate(cls, w: int, h: int, cam: abi.Camera, device="cuda") -> "DiffViewBuffers":
        dev = torch.device(device)
        cam_t = torch.from_numpy(np.frombuffer(C.string_at(C.addressof(cam), C.sizeof(cam)), np.uint8).copy()).to(dev)
        return cls(w, h, cam_t, torch.zeros(w * h, dtype=torch.int64, device=dev))

    def ids(self) -> np.ndarray:
        lo = (self.depth_id.cpu().numpy().view(np.uint64) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        return np.where(lo == 0, np.uint32(0xFFFFFFFF), lo - np.uint32(1)).astype(np.uint32)


def _views(views, rgb=None, target=None, grad=None):
    arr = (abi.DiffView * len(views))()
    for i, v in enumerate(views):
        arr[i].camera_buffer = _ptr(v.camera)
        arr[i].width, arr[i].height = v.width, v.height
        arr[i].depth_id = _ptr(v.depth_id)
        arr[i].rgb = _ptr(rgb[i]) if rgb is not None else 0
        arr[i].target = _ptr(target[i]) if target is not None else 0
        arr[i].grad_rgb = _ptr(grad[i]) if grad is not None else 0
    return arr


def forward(r: Renderer, scene: DiffScene, views, rgb_out, positions=None, colors=None, texture=None,
            stream=None) -> None:
    """Renders linear RGB (float32 [H*W*3] per view) into rgb_out[i]."""
    s = scene.struct(positions, colors, texture)
    arr = _views(views, rgb=rgb_out)
    abi.check(r.lib.vkgv_diff_forward(r.ctx, C.byref(s), arr, len(views), _stream_handle(stream)), r.ctx)


def backward(r: Renderer, scene: DiffScene, views, grad_positions=None, grad_colors=None, grad_texture=None,
             targets=None, grad_rgb=None, scale: float = 1.0, loss=None, positions=None, colors=None,
             texture=None, stream=None) -> None:
    """Accumulates parameter gradients; either MSE `targets` (with `scale`
    and an optional float32 `loss` accumulator) or upstream `grad_rgb`."""
    s = scene.struct(positions, colors, texture)
    arr = _views(views, target=targets, grad=grad_rgb if targets is None else None)
    abi.check(r.lib.vkgv_diff_backward(r.ctx, C.byref(s), arr, len(views), float(scale), _ptr(loss),
                                       _ptr(grad_positions), _ptr(grad_colors), _ptr(grad_texture),
                                       _stream_handle(stream)), r.ctx)


def capture_step(r: Renderer, scene: DiffScene, views, rgb_out=None, targets=None, grad_rgb=None,
                 grad_positions=None, grad_colors=None, grad_texture=None, scale: float = 1.0, loss=None,
                 passes: int = abi.DIFF_ZERO_GRADS | abi.DIFF_FORWARD | abi.DIFF_BACKWARD) -> Graph:
    """Captures zeroing, forward and backward (as selected by `passes`) into
    one CUDA graph; tensors are baked in by address, their contents may
    change between launches."""
    s = scene.struct()
    arr = _views(views, rgb=rgb_out, target=targets, grad=grad_rgb if targets is None else None)
    h = C.c_void_p()
    abi.check(r.lib.vkgv_diff_graph_capture(r.ctx, C.byref(s), arr, len(views), int(passes), float(scale),
                                            _ptr(loss), _ptr(grad_positions), _ptr(grad_colors),
                                            _ptr(grad_texture), C.byref(h)), r.ctx)
    return Graph(r, h.value, keep=(scene, views, rgb_out, targets, grad_rgb, grad_positions, grad_colors,
                                   grad_texture, loss))
