"""glTF 2.0 assets into the renderer's layout (``vkgv_gltf_*``).

``load`` returns the ``HostScene`` (one primitive per glTF primitive, with
meshlets; materials with index 0 the glTF default) and the ``HostWorld``
(node tree, meshes as primitive lists, animations) of an asset, as
AssetLoadTask + World::addAsset do (src/vk_gltf_viewer/assets.cpp:288-552,
world.cpp:9-80).  ``device_scene`` uploads them and has the world kernels
write the transforms and the draw list.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi, scene
from .world import NODE_DTYPE, DeviceWorld, HostWorld, Sampler


def load(path, texture_references: bool = False, images: bool = False,
         renderer=None) -> tuple[scene.HostScene, HostWorld]:
    """With `images`, the base-colour textures are decoded too (PNG on the
    host, DDS block formats on the renderer's device) into the scene's
    texture table, indexed like the glTF textures, and the materials keep
    their texture references."""
    lib = abi.load()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    flags = (abi.GLTF_TEXTURE_REFERENCES if (texture_references or images) else 0) | (abi.GLTF_IMAGES if images else 0)
    rc = lib.vkgv_gltf_load(str(Path(path)).encode(), flags, C.byref(h), err, len(err))
    if rc != abi.OK:
        raise abi.VkgvError(rc, err.value.decode(errors="replace"))
    try:
        info = abi.GltfInfo()
        abi.check(lib.vkgv_gltf_get_info(h, C.byref(info)))
        meshes, prim_materials, counts = [], [], []
        for i in range(info.primitive_count):
            p = abi.GltfPrimitive()
            abi.check(lib.vkgv_gltf_get_primitive(h, i, C.byref(p)))
            meshes.append(scene._mesh_from_handle(p.mesh, owned=False))
            prim_materials.append(int(p.material_index))
            counts.append(int(p.meshlet_count))
        mats = np.zeros(info.material_count, scene.MATERIAL_DTYPE)
        abi.check(lib.vkgv_gltf_get_materials(h, mats.ctypes.data, info.material_count))
        d = abi.WorldDesc()
        abi.check(lib.vkgv_gltf_get_world(h, C.byref(d)))
        world = _world_from_desc(d)
        textures = []
        if images:
            from . import texture
            for t in range(info.texture_count):
                gi = abi.GltfImage()
                abi.check(lib.vkgv_gltf_get_texture_image(h, t, C.byref(gi)))
                if not gi.data:
                    rgba = np.full((1, 1, 4), 255, np.uint8)  # a texture without an image samples white
                else:
                    rgba = texture.load_image(C.string_at(gi.data, gi.size), gi.kind, renderer)
                fmt = abi.TEXTURE_RGB32F if rgba.dtype == np.float32 else abi.TEXTURE_RGBA8  # BC6H: linear float RGB
                textures.append(scene.Texture(np.ascontiguousarray(rgba), fmt))
    finally:
        lib.vkgv_gltf_free(h)
    draws = world.draw_list()
    t = len(world.visits())
    transforms = np.tile(scene.to_column_major(np.eye(4)), (max(t, 0), 1)).reshape(t, 16)
    host = scene.HostScene(meshes=meshes, prim_materials=prim_materials, materials=mats, transforms=transforms,
                           node_meshes=[], draws=draws, textures=textures)
    return host, world


def meshopt_decode(data: bytes, count: int, stride: int, mode: int,
                   filter: int = abi.MESHOPT_FILTER_NONE) -> np.ndarray:
    """One EXT_meshopt_compression bufferView decoded (and filtered) into
    ``count * stride`` bytes, as MeshoptDecompressor::ExecuteRange does per
    view (src/vk_gltf_viewer/assets.cpp:111-166).  Raises ``VkgvError`` for a
    stream that does not decode to exactly its declared size."""
    lib = abi.load()
    out = np.empty(count * stride, np.uint8)
    src = bytes(data)
    abi.check(lib.vkgv_meshopt_decode(out.ctypes.data, count, stride, src, len(src), mode, filter))
    return out


def _copy(ptr, n, dtype):
    dtype = np.dtype(dtype)
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.frombuffer(C.string_at(ptr, n * dtype.itemsize), dtype, n).copy()


def _world_from_desc(d: abi.WorldDesc) -> HostWorld:
    nodes = _copy(d.nodes, d.node_count, NODE_DTYPE)
    offs = _copy(d.mesh_offsets, d.mesh_count + 1, np.uint32)
    prims = _copy(d.mesh_primitives, int(offs[-1]) if offs.size else 0, np.uint32)
    mesh_primitives = [[int(x) for x in prims[offs[m]:offs[m + 1]]] for m in range(d.mesh_count)]
    samplers = []
    sd = (abi.AnimSampler * max(1, d.sampler_count)).from_address(d.samplers) if d.sampler_count else []
    for i in range(d.sampler_count):
        s = sd[i]
        inp = _copy(s.input, s.input_count, np.float32)
        out = _copy(s.output, s.output_count * s.components, np.float32).reshape(s.output_count, s.components)
        samplers.append(Sampler(inp, out, int(s.interpolation)))
    channels = _copy(d.channels, d.channel_count * 4, np.uint32).reshape(-1, 4)
    return HostWorld(nodes=nodes, children=_copy(d.children, d.child_count, np.uint32),
                     roots=_copy(d.roots, d.root_count, np.uint32), mesh_primitives=mesh_primitives,
                     primitive_meshlet_counts=_copy(d.primitive_meshlet_counts, d.primitive_count, np.uint32),
                     samplers=samplers, channels=channels)


def device_scene(renderer, host: scene.HostScene, world: HostWorld, animation_time: float = 0.0, device="cuda"):
    """Uploads an imported asset and lets the world kernels write its
    transforms (at `animation_time`) and draw list on the device.  Returns
    (DeviceScene, DeviceWorld); call DeviceWorld.update_transforms on the
    scene's transform buffer each frame to animate it."""
    from .renderer import DeviceScene

    dev = DeviceScene(host, device)
    dw = DeviceWorld(renderer, world)
    if dw.transform_count:
        dw.update_transforms(animation_time, dev.transforms)
    if dw.draw_count:
        dw.build_draws(dev.draws)
    return dev, dw
