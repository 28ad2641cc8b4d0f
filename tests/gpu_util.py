"""Shared setup for the GPU parity tests: one host scene feeds both the CUDA
path (through the C ABI) and the CPU oracle."""
from __future__ import annotations

import numpy as np
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, scene
from vk_gltf_viewer_gb300.renderer import DeviceScene, ViewBuffers

ORACLE_FLAGS = {
    abi.CULL_FRUSTUM: ob.CULL_FRUSTUM, abi.CULL_OCCLUSION: ob.CULL_OCCLUSION, abi.CULL_TWO_PASS: ob.CULL_TWO_PASS,
    abi.CULL_CONE: ob.CULL_CONE, abi.CULL_OCCLUSION_FINE: ob.CULL_OCCLUSION_FINE,
    abi.RESOLVE_FLAT: ob.RESOLVE_FLAT, abi.RESOLVE_TEXTURED: ob.RESOLVE_TEXTURED,
    abi.BUILD_PYRAMID: ob.BUILD_PYRAMID,
}


def oracle_flags(flags: int) -> int:
    out = 0
    for k, v in ORACLE_FLAGS.items():
        if flags & k:
            out |= v
    return out


class Pair:
    """A host scene on the device and in the oracle."""

    def __init__(self, host: scene.HostScene):
        self.host = host
        self.dev = DeviceScene(host, "cuda")
        self.orc = ob.OracleScene(host)


def view(pair: Pair, cam, w: int, h: int, prev: np.ndarray | None = None) -> ViewBuffers:
    v = ViewBuffers.allocate(w, h, cam, pair.host.draw_count, prev_pyramid=prev is not None)
    if prev is not None:
        v.prev_pyramid.copy_(torch.from_numpy(prev).cuda())
    return v


def u64(t: torch.Tensor) -> np.ndarray:
    return t.cpu().numpy().view(np.uint64)


def u32(t: torch.Tensor) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def rgba_close(a: np.ndarray, b: np.ndarray, tol: int = 1) -> tuple[bool, int]:
    """Per-channel |a - b| <= tol (1/255 for the resolve)."""
    ca = a.view(np.uint8).reshape(-1, 4).astype(np.int32)
    cb = b.view(np.uint8).reshape(-1, 4).astype(np.int32)
    d = np.abs(ca - cb).max(axis=1)
    return bool((d <= tol).all()), int((d > tol).sum())


def orbit_cameras(n: int, radius: float, w: int, h: int, seed: int, centre=(0.0, 0.0, 0.0), fovy: float = 60.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        eye = np.asarray(centre) + radius * v
        out.append(scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), fovy, w / h))
    return out


def small_grid(tex: int = 64, grid=(4, 4, 2)) -> scene.HostScene:
    return scene.scene_torus_grid(texture_size=tex, grid=grid)
