"""The node tree of a scene and its per-frame device buffers.

Mirrors ``World`` (src/vk_gltf_viewer/world.cpp): ``HostWorld`` holds the
merged node, mesh and animation tables that ``World::addAsset`` builds, and
``DeviceWorld`` wraps ``vkgv_world_*``: ``update_transforms`` is
``World::updateTransformBuffer`` and ``build_draws`` is
``World::rebuildDrawBuffer``, both written by CUDA kernels straight into the
scene's device buffers.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import abi, scene
from .renderer import _stream_handle

NODE_DTYPE = np.dtype({"names": ["translation", "rotation", "scale", "mesh_index", "first_child", "child_count"],
                       "formats": [("<f4", 3), ("<f4", 4), ("<f4", 3), "<u4", "<u4", "<u4"],
                       "offsets": [0, 12, 28, 40, 44, 48], "itemsize": 52})


@dataclass
class Sampler:
    """An animation sampler (assets.hpp:37-47)."""
    input: np.ndarray          # float32 keyframe times, ascending
    output: np.ndarray         # float32 (output_count, components)
    interpolation: int         # abi.INTERP_*

    @property
    def components(self) -> int:
        return int(self.output.shape[1])


@dataclass
class HostWorld:
    """Node tree (DecomposeNodeMatrices TRS), meshes as primitive lists, the
    primitives' meshlet counts and the animations' samplers and channels."""
    nodes: np.ndarray                       # NODE_DTYPE
    children: np.ndarray                    # uint32
    roots: np.ndarray                       # uint32, scenes[0].nodeIndices
    mesh_primitives: list[list[int]]
    primitive_meshlet_counts: np.ndarray    # uint32
    samplers: list[Sampler] = field(default_factory=list)
    channels: np.ndarray | None = None      # (C, 4) uint32: sampler, node, path, 0

    def __post_init__(self):
        self.children = np.ascontiguousarray(self.children, np.uint32)
        self.roots = np.ascontiguousarray(self.roots, np.uint32)
        self.primitive_meshlet_counts = np.ascontiguousarray(self.primitive_meshlet_counts, np.uint32)
        if self.channels is None:
            self.channels = np.zeros((0, 4), np.uint32)
        self.channels = np.ascontiguousarray(self.channels, np.uint32).reshape(-1, 4)
        offs = np.zeros(len(self.mesh_primitives) + 1, np.uint32)
        offs[1:] = np.cumsum([len(p) for p in self.mesh_primitives])
        self.mesh_offsets = offs
        flat = [p for prims in self.mesh_primitives for p in prims]
        self.mesh_primitive_array = np.asarray(flat if flat else [0], np.uint32)
        self._samplers_c = (abi.AnimSampler * max(1, len(self.samplers)))()
        self._sampler_keep = []
        for i, s in enumerate(self.samplers):
            inp = np.ascontiguousarray(s.input, np.float32)
            out = np.ascontiguousarray(s.output, np.float32)
            self._sampler_keep += [inp, out]
            self._samplers_c[i] = abi.AnimSampler(inp.ctypes.data, out.ctypes.data, inp.size, out.shape[0],
                                                  s.interpolation, out.shape[1])

    def desc_fields(self) -> dict:
        """Field values shared by vkgv_world_desc and the oracle's orc_world."""
        n = self.nodes
        return dict(nodes=n.ctypes.data, node_count=n.size, child_count=self.children.size,
                    children=self.children.ctypes.data, roots=self.roots.ctypes.data, root_count=self.roots.size,
                    mesh_count=len(self.mesh_primitives), mesh_offsets=self.mesh_offsets.ctypes.data,
                    mesh_primitives=self.mesh_primitive_array.ctypes.data,
                    primitive_meshlet_counts=self.primitive_meshlet_counts.ctypes.data,
                    primitive_count=self.primitive_meshlet_counts.size, sampler_count=len(self.samplers),
                    samplers=C.addressof(self._samplers_c), channels=self.channels.ctypes.data,
                    channel_count=self.channels.shape[0])

    def desc(self) -> abi.WorldDesc:
        return abi.WorldDesc(**self.desc_fields())

    def visits(self) -> list[int]:
        """Nodes with a mesh in depth-first order from the roots: entry i is
        the node of transform slot i (World::iterateNode)."""
        out = []
        stack = [int(r) for r in self.roots[::-1]]
        depth_stack = [0] * len(stack)
        while stack:
            n, d = stack.pop(), depth_stack.pop()
            if d >= abi.MAX_NODE_DEPTH:
                raise ValueError("node tree deeper than 64 (or cyclic)")
            node = self.nodes[n]
            if node["mesh_index"] != abi.INVALID_HANDLE:
                out.append(n)
            f, c = int(node["first_child"]), int(node["child_count"])
            kids = [int(x) for x in self.children[f:f + c][::-1]]
            stack.extend(kids)
            depth_stack.extend([d + 1] * len(kids))
        return out

    def draw_list(self) -> np.ndarray:
        """World::rebuildDrawBuffer on the host: (D, 3) uint32 {primitive,
        meshlet, transform} (the device builds the same list)."""
        parts = []
        for slot, n in enumerate(self.visits()):
            m = int(self.nodes[n]["mesh_index"])
            for p in self.mesh_primitives[m]:
                k = int(self.primitive_meshlet_counts[p])
                if k:
                    d = np.empty((k, 3), np.uint32)
                    d[:, 0], d[:, 1], d[:, 2] = p, np.arange(k, dtype=np.uint32), slot
                    parts.append(d)
        return np.ascontiguousarray(np.concatenate(parts)) if parts else np.zeros((0, 3), np.uint32)

    @property
    def meshlet_draw_count(self) -> int:
        """Draw count by a host walk of the tree (the plan's own count is
        DeviceWorld.draw_count)."""
        counts = [int(sum(int(self.primitive_meshlet_counts[p]) for p in prims)) for prims in self.mesh_primitives]
        total = 0
        stack = list(self.roots[::-1])
        while stack:
            n = int(stack.pop())
            node = self.nodes[n]
            if node["mesh_index"] != abi.INVALID_HANDLE:
                total += counts[int(node["mesh_index"])]
            f, c = int(node["first_child"]), int(node["child_count"])
            stack.extend(int(x) for x in self.children[f:f + c][::-1])
        return total


def make_nodes(n: int) -> np.ndarray:
    nodes = np.zeros(n, NODE_DTYPE)
    nodes["rotation"][:, 3] = 1.0
    nodes["scale"] = 1.0
    nodes["mesh_index"] = abi.INVALID_HANDLE
    return nodes


def quat_axis_angle(axis, angle: float) -> np.ndarray:
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    s = math.sin(angle / 2)
    return np.array([a[0] * s, a[1] * s, a[2] * s, math.cos(angle / 2)], np.float32)


def grid_world(mesh_meshlets: int, position_scale: float = 1.0, seed: int = 7, grid=scene.GRID,
               animated: bool = True) -> HostWorld:
    """The torus grid as a node tree: a root, one node per layer (y) and one
    torus node per grid cell under its layer (translation, seeded yaw,
    quantisation scale), in the instance order of scene_torus_grid.  With
    `animated`, seeded channels of every kind: layers sway (LINEAR rotation),
    a quarter of the tori bob (CUBICSPLINE translation), an eighth spin
    (LINEAR rotation through 120-degree steps), a sixteenth pulse (STEP
    scale), some drift (LINEAR translation) or wobble (CUBICSPLINE rotation);
    plus one weights channel and one untargeted channel, which do nothing."""
    gx, gz, gy = grid
    rng = np.random.default_rng(seed)
    per_layer = gx * gz
    n = 1 + gy + gy * per_layer
    nodes = make_nodes(n)
    children = []
    nodes[0]["first_child"], nodes[0]["child_count"] = 0, gy
    children += list(range(1, 1 + gy))
    for k in range(gy):
        layer = 1 + k
        nodes[layer]["translation"] = (0.0, k * scene.SPACING, 0.0)
        nodes[layer]["first_child"], nodes[layer]["child_count"] = len(children), per_layer
        first = 1 + gy + k * per_layer
        children += list(range(first, first + per_layer))
        for j in range(gz):
            for i in range(gx):
                t = first + j * gx + i
                yaw = rng.uniform(0, 2 * math.pi)
                nodes[t]["translation"] = (i * scene.SPACING, 0.0, j * scene.SPACING)
                nodes[t]["rotation"] = quat_axis_angle((0, 1, 0), yaw)
                nodes[t]["scale"] = position_scale
                nodes[t]["mesh_index"] = 0
    samplers: list[Sampler] = []
    channels = []
    if animated:
        times4 = np.array([0.0, 1.0, 2.5, 4.0], np.float32)
        for k in range(gy):
            angles = rng.uniform(-0.08, 0.08, 4)
            out = np.stack([quat_axis_angle((0, 1, 0), a) for a in angles])
            samplers.append(Sampler(times4, out, abi.INTERP_LINEAR))
            channels.append((len(samplers) - 1, 1 + k, abi.PATH_ROTATION, 0))
        tori = np.arange(1 + gy, n)
        pick = rng.permutation(tori)
        q = len(tori)
        for t in pick[: q // 4]:
            base = nodes[t]["translation"].astype(np.float32)
            keys = np.sort(rng.uniform(0.0, 3.0, 5)).astype(np.float32)
            keys[0] = 0.0
            vals = np.repeat(base[None, :], 5, 0)
            vals[:, 1] += rng.uniform(-0.3, 0.3, 5).astype(np.float32)
            tang = rng.uniform(-0.5, 0.5, (5, 2, 3)).astype(np.float32)
            out = np.concatenate([tang[:, :1], vals[:, None], tang[:, 1:]], 1).reshape(15, 3)
            samplers.append(Sampler(keys, out, abi.INTERP_CUBICSPLINE))
            channels.append((len(samplers) - 1, int(t), abi.PATH_TRANSLATION, 0))
        spin_keys = np.array([0.0, 0.7, 1.4, 2.1], np.float32)
        for t in pick[q // 4: q // 4 + q // 8]:
            yaw0 = rng.uniform(0, 2 * math.pi)
            out = np.stack([quat_axis_angle((0, 1, 0), yaw0 + a) for a in (0.0, 2.0944, 4.1888, 6.2832)])
            samplers.append(Sampler(spin_keys, out, abi.INTERP_LINEAR))
            channels.append((len(samplers) - 1, int(t), abi.PATH_ROTATION, 0))
        for t in pick[q // 4 + q // 8: q // 4 + q // 8 + q // 16]:
            s0 = float(nodes[t]["scale"][0])
            out = (np.array([1.0, 1.15, 0.9], np.float32)[:, None] * s0).repeat(3, 1)
            samplers.append(Sampler(np.array([0.0, 0.5, 1.0], np.float32), out, abi.INTERP_STEP))
            channels.append((len(samplers) - 1, int(t), abi.PATH_SCALE, 0))
        rest = pick[q // 4 + q // 8 + q // 16:]
        for t in rest[: q // 16]:
            base = nodes[t]["translation"].astype(np.float32)
            out = np.stack([base, base + rng.uniform(-0.2, 0.2, 3).astype(np.float32)])
            samplers.append(Sampler(np.array([0.0, 2.0], np.float32), out, abi.INTERP_LINEAR))
            channels.append((len(samplers) - 1, int(t), abi.PATH_TRANSLATION, 0))
        for t in rest[q // 16: q // 16 + q // 32]:
            q0 = nodes[t]["rotation"].astype(np.float32)
            keys = np.array([0.0, 1.0, 2.0], np.float32)
            vals = np.stack([q0, quat_axis_angle(rng.normal(size=3), 0.4), q0])
            tang = rng.uniform(-0.2, 0.2, (3, 2, 4)).astype(np.float32)
            out = np.concatenate([tang[:, :1], vals[:, None], tang[:, 1:]], 1).reshape(9, 4)
            samplers.append(Sampler(keys, out, abi.INTERP_CUBICSPLINE))
            channels.append((len(samplers) - 1, int(t), abi.PATH_ROTATION, 0))
        # a weights channel and a channel without a target node are ignored
        channels.append((0, 1, abi.PATH_WEIGHTS, 0))
        channels.append((0, abi.INVALID_HANDLE, abi.PATH_ROTATION, 0))
    return HostWorld(nodes=nodes, children=np.asarray(children, np.uint32), roots=np.array([0], np.uint32),
                     mesh_primitives=[[0]], primitive_meshlet_counts=np.array([mesh_meshlets], np.uint32),
                     samplers=samplers, channels=np.asarray(channels, np.uint32).reshape(-1, 4))


class DeviceWorld:
    """A planned world on one context (``vkgv_world_create``)."""

    def __init__(self, renderer, host: HostWorld):
        self.renderer = renderer
        self.host = host
        self.lib = abi.load()
        self._desc = host.desc()
        h = C.c_void_p()
        abi.check(self.lib.vkgv_world_create(renderer.ctx, C.byref(self._desc), C.byref(h)), renderer.ctx)
        self.handle = h
        t, d = C.c_uint32(), C.c_uint64()
        abi.check(self.lib.vkgv_world_info(self.handle, C.byref(t), C.byref(d)))
        self.transform_count = int(t.value)
        self.draw_count = int(d.value)

    def update_transforms(self, animation_time: float, transforms: torch.Tensor, stream=None) -> None:
        """World::updateTransformBuffer into `transforms` (float32, 16 per slot)."""
        if transforms.numel() * transforms.element_size() < 64 * self.transform_count:
            raise ValueError("transform buffer too small")
        abi.check(self.lib.vkgv_world_update_transforms(self.renderer.ctx, self.handle, float(animation_time),
                                                        transforms.data_ptr(), _stream_handle(stream)), self.renderer.ctx)

    def build_draws(self, draws: torch.Tensor, stream=None) -> None:
        """World::rebuildDrawBuffer into `draws` (3 words per MeshletDraw)."""
        abi.check(self.lib.vkgv_world_build_draws(self.renderer.ctx, self.handle, draws.data_ptr(),
                                                  draws.numel() * draws.element_size() // 12, _stream_handle(stream)),
                  self.renderer.ctx)

    def close(self) -> None:
        if self.handle:
            self.lib.vkgv_world_destroy(self.handle)
            self.handle = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
