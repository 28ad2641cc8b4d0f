"""Launch-shape autotuner for the raster: picks the bin size {8, 16, 32} and
meshlets per CTA {1, 2, 4} for a workload on this GPU.

The sweep itself is native (vkgv_autotune: one context and one captured
frame graph per candidate, timed with CUDA events).  Results are cached in a
JSON file keyed by GPU name, SM count and a workload key (triangles, draws,
flags, view count and resolutions), so a workload is swept once per GPU
model.  The cache path is $VKGV_AUTOTUNE_CACHE, else
~/.cache/vk_gltf_viewer_gb300/autotune.json.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import torch

from .renderer import DeviceScene, Renderer, ViewBuffers


def cache_path() -> Path:
    env = os.environ.get("VKGV_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "vk_gltf_viewer_gb300" / "autotune.json"


def device_key(device: int) -> str:
    p = torch.cuda.get_device_properties(device)
    return f"{p.name}|sm{p.multi_processor_count}|cc{p.major}.{p.minor}"


def workload_key(scene: DeviceScene, views: list[ViewBuffers], flags: int) -> str:
    sizes = ",".join(f"{v.width}x{v.height}" for v in views)
    digest = hashlib.sha1(sizes.encode()).hexdigest()[:12]
    return (f"tris={scene.host.triangle_count}|draws={scene.draw_count}|flags={flags:#x}|views={len(views)}"
            f"|px={sum(v.width * v.height for v in views)}|sizes={digest}")


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def tune(r: Renderer, scene: DeviceScene, views: list[ViewBuffers], flags: int, launches: int = 3,
         path: Path | None = None, force: bool = False) -> dict:
    """Returns {"bin_size", "meshlets_per_cta", "table", "cached", "key"} for
    this workload, sweeping (and caching) unless a cached entry exists."""
    path = path or cache_path()
    key = device_key(r.device) + "||" + workload_key(scene, views, flags)
    cache = _load(path)
    if not force and key in cache:
        out = dict(cache[key])
        out.update(cached=True, key=key)
        return out
    table, (bin_size, split) = r.sweep(scene, views, flags, launches)
    entry = {"bin_size": bin_size, "meshlets_per_cta": split,
             "table": [{"bin_size": b, "meshlets_per_cta": m, "ms_per_launch": ms} for b, m, ms in table]}
    cache = _load(path)
    cache[key] = entry
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        tmp.replace(path)
    except OSError:
        pass
    out = dict(entry)
    out.update(cached=False, key=key)
    return out


def tuned_renderer(r: Renderer, scene: DeviceScene, views: list[ViewBuffers], flags: int, **kw):
    """A Renderer on r's device configured with the tuned launch shape, and
    the tuning record."""
    rec = tune(r, scene, views, flags, **kw)
    return Renderer(r.device, bin_size=rec["bin_size"], meshlets_per_cta=rec["meshlets_per_cta"],
                    big_capacity=r.big_capacity), rec
