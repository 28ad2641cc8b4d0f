"""A small glTF 2.0 writer: accessors (float or KHR_mesh_quantization
integers, strided or sparse), meshes, materials with KHR_texture_transform,
nodes (TRS or matrix), scenes and animations, written as .glb or as .gltf
with a base64 data URI or an external .bin.  ``write_world`` exports a scene
built in this package (its primitives and node tree) so that it can be read
back through the importer."""
from __future__ import annotations

import base64
import json
import struct
from pathlib import Path

import numpy as np

FLOAT, BYTE, UBYTE, SHORT, USHORT, UINT = 5126, 5120, 5121, 5122, 5123, 5125
_TYPES = {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4", 16: "MAT4"}
_CT = {np.dtype(np.float32): FLOAT, np.dtype(np.int8): BYTE, np.dtype(np.uint8): UBYTE,
       np.dtype(np.int16): SHORT, np.dtype(np.uint16): USHORT, np.dtype(np.uint32): UINT}


class Builder:
    def __init__(self):
        self.bin = bytearray()
        self.gltf = {"asset": {"version": "2.0", "generator": "vkgv tests"}, "buffers": [], "bufferViews": [],
                     "accessors": []}

    def _view(self, data: bytes, stride: int | None = None) -> int:
        while len(self.bin) % 4:
            self.bin.append(0)
        view = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            view["byteStride"] = stride
        self.bin += data
        self.gltf["bufferViews"].append(view)
        return len(self.gltf["bufferViews"]) - 1

    def accessor(self, arr: np.ndarray, normalized: bool = False, minmax: bool = False, stride: int | None = None,
                 sparse: tuple[np.ndarray, np.ndarray] | None = None) -> int:
        """arr: (count, ncomp) or (count,).  With `stride`, elements are
        interleaved with padding up to `stride` bytes."""
        a = np.ascontiguousarray(arr)
        count = a.shape[0]
        ncomp = 1 if a.ndim == 1 else a.shape[1]
        raw = a.tobytes()
        if stride:
            elem = a.dtype.itemsize * ncomp
            buf = bytearray(stride * count)
            for i in range(count):
                buf[i * stride:i * stride + elem] = raw[i * elem:(i + 1) * elem]
            raw = bytes(buf)
        acc = {"bufferView": self._view(raw, stride), "componentType": _CT[a.dtype], "count": count,
               "type": _TYPES[ncomp]}
        if normalized:
            acc["normalized"] = True
        if minmax:
            acc["min"] = [float(x) for x in a.reshape(count, ncomp).min(0)]
            acc["max"] = [float(x) for x in a.reshape(count, ncomp).max(0)]
        if sparse is not None:
            idx, vals = sparse
            acc["sparse"] = {"count": int(idx.size),
                             "indices": {"bufferView": self._view(np.ascontiguousarray(idx, np.uint32).tobytes()),
                                         "componentType": UINT},
                             "values": {"bufferView": self._view(np.ascontiguousarray(vals, a.dtype).tobytes())}}
        self.gltf["accessors"].append(acc)
        return len(self.gltf["accessors"]) - 1

    def add(self, key: str, obj: dict) -> int:
        self.gltf.setdefault(key, []).append(obj)
        return len(self.gltf[key]) - 1

    def _finish(self, uri: str | None):
        while len(self.bin) % 4:
            self.bin.append(0)
        buf = {"byteLength": len(self.bin)}
        if uri is not None:
            buf["uri"] = uri
        self.gltf["buffers"] = [buf]

    def write_glb(self, path: Path) -> Path:
        self._finish(None)
        js = json.dumps(self.gltf).encode()
        js += b" " * (-len(js) % 4)
        total = 12 + 8 + len(js) + 8 + len(self.bin)
        out = struct.pack("<III", 0x46546C67, 2, total) + struct.pack("<II", len(js), 0x4E4F534A) + js
        out += struct.pack("<II", len(self.bin), 0x004E4942) + bytes(self.bin)
        Path(path).write_bytes(out)
        return Path(path)

    def write_gltf(self, path: Path, external: str | None = None) -> Path:
        """A .gltf with the buffer as a data URI, or in `external` (a file
        name next to it, written percent-encoded in the URI)."""
        path = Path(path)
        if external is None:
            self._finish("data:application/octet-stream;base64," + base64.b64encode(bytes(self.bin)).decode())
        else:
            from urllib.parse import quote
            self._finish(quote(external))
            (path.parent / external).write_bytes(bytes(self.bin))
        path.write_text(json.dumps(self.gltf, indent=1, ensure_ascii=False))
        return path


def quantize_i16(pos: np.ndarray) -> tuple[np.ndarray, float]:
    """Positions as int16-normalised values q with pos ~= q / 32767 * s."""
    s = float(np.abs(pos).max())
    q = np.round(pos / s * 32767.0).astype(np.int16)
    return q, s


_PATHS = {1: "translation", 2: "rotation", 3: "scale", 4: "weights"}
_INTERP = {0: "LINEAR", 1: "STEP", 2: "CUBICSPLINE"}


def write_world(path, meshes, world, material: dict | None = None) -> Path:
    """One glTF mesh per primitive (positions, UVs when present, uint32
    indices, material 0), the world's nodes, first scene and animations, as
    a .glb.  `material` is the glTF material dict (default: white)."""
    b = Builder()
    for m in meshes:
        attrs = {"POSITION": b.accessor(np.asarray(m.positions, np.float32))}
        if m.uvs is not None:
            attrs["TEXCOORD_0"] = b.accessor(np.asarray(m.uvs, np.float32))
        b.add("meshes", {"primitives": [{"attributes": attrs, "material": 0,
                                         "indices": b.accessor(np.asarray(m.indices, np.uint32).reshape(-1))}]})
    b.add("materials", material if material is not None else {})
    for n in world.nodes:
        node = {"translation": [float(x) for x in n["translation"]],
                "rotation": [float(x) for x in n["rotation"]], "scale": [float(x) for x in n["scale"]]}
        if n["mesh_index"] != 0xFFFFFFFF:
            node["mesh"] = int(n["mesh_index"])
        f, c = int(n["first_child"]), int(n["child_count"])
        if c:
            node["children"] = [int(x) for x in world.children[f:f + c]]
        b.add("nodes", node)
    b.gltf["scenes"] = [{"nodes": [int(r) for r in world.roots]}]
    if world.samplers:
        samplers = [{"input": b.accessor(s.input), "output": b.accessor(s.output),
                     "interpolation": _INTERP[s.interpolation]} for s in world.samplers]
        channels = []
        for sm, node, kind, _ in world.channels.tolist():
            target = {"path": _PATHS[kind]}
            if node != 0xFFFFFFFF:
                target["node"] = node
            channels.append({"sampler": sm, "target": target})
        b.add("animations", {"samplers": samplers, "channels": channels})
    return b.write_glb(path)
