"""A small glTF 2.0 writer: accessors (float or KHR_mesh_quantization
integers, strided or sparse), meshes, materials with KHR_texture_transform,
nodes (TRS or matrix), scenes and animations, EXT_meshopt_compression
buffer views (streams encoded by the caller), written as .glb or as .gltf
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
        self.fallback = 0  # bytes of the EXT_meshopt_compression fallback buffer (no data)
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

    def meshopt_view(self, stream: bytes, count: int, stride: int, mode: str, filter: str = "NONE",
                     byte_stride: int | None = None) -> int:
        """A bufferView of ``count * stride`` bytes stored as the
        EXT_meshopt_compression `stream` (encoded by the caller) in buffer 0;
        the view itself lies in a fallback buffer without data."""
        while len(self.bin) % 4:
            self.bin.append(0)
        ext = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(stream), "byteStride": stride,
               "count": count, "mode": mode}
        if filter != "NONE":
            ext["filter"] = filter
        self.bin += stream
        view = {"buffer": 1, "byteOffset": self.fallback, "byteLength": count * stride,
                "extensions": {"EXT_meshopt_compression": ext}}
        if byte_stride:
            view["byteStride"] = byte_stride
        self.fallback += (count * stride + 3) // 4 * 4
        self.gltf["bufferViews"].append(view)
        return len(self.gltf["bufferViews"]) - 1

    def view_accessor(self, view: int, dtype, count: int, ncomp: int, normalized: bool = False) -> int:
        acc = {"bufferView": view, "componentType": _CT[np.dtype(dtype)], "count": count, "type": _TYPES[ncomp]}
        if normalized:
            acc["normalized"] = True
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
        if self.fallback:
            self.gltf["buffers"].append({"byteLength": self.fallback,
                                         "extensions": {"EXT_meshopt_compression": {"fallback": True}}})
            used = self.gltf.setdefault("extensionsUsed", [])
            if "EXT_meshopt_compression" not in used:
                used.append("EXT_meshopt_compression")

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
        while len(self.bin) % 4:  # before the URI or file is made from it
            self.bin.append(0)
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


# ------------------------------------------------- EXT_meshopt_compression

def meshopt_encode_attributes(data: np.ndarray) -> bytes:
    """(count, stride) uint8 vertex records -> an EXT_meshopt_compression
    ATTRIBUTES stream: per block and byte column, zig-zag deltas against the
    previous vertex (the first against a zero baseline), each group of 16 in
    its smallest mode (0 / 2 / 4 / 8 bits with escapes)."""
    v = np.ascontiguousarray(data, np.uint8)
    count, stride = v.shape
    assert stride % 4 == 0 and 0 < stride <= 256
    block = min((8192 // stride) // 16 * 16, 256)
    prev = np.concatenate([np.zeros((1, stride), np.uint8), v[:-1]]) if count else v
    d = (v.astype(np.int16) - prev.astype(np.int16)) & 0xFF
    sd = np.where(d >= 128, d - 256, d)
    zz = np.where(sd >= 0, 2 * sd, -2 * sd - 1).astype(np.uint8)
    out = [b"\xa0"]
    for first in range(0, count, block):
        n = min(block, count - first)
        groups = (n + 15) // 16
        z = np.zeros((stride, groups * 16), np.uint8)
        z[:, :n] = zz[first:first + n].T
        g = z.reshape(stride * groups, 16)  # rows: column-major groups
        esc2, esc4 = (g >= 3).sum(1), (g >= 15).sum(1)
        sizes = np.stack([np.where(g.any(1), 1 << 20, 0), 4 + esc2, 8 + esc4, np.full(len(g), 16)], 1)
        mode = sizes.argmin(1)
        length = sizes[np.arange(len(g)), mode]
        payload = np.zeros((len(g), 24), np.uint8)
        c2 = np.minimum(g, 3).reshape(-1, 4, 4)
        payload[mode == 1, :4] = ((c2[:, :, 0] << 6) | (c2[:, :, 1] << 4) | (c2[:, :, 2] << 2) | c2[:, :, 3])[mode == 1]
        c4 = np.minimum(g, 15).reshape(-1, 8, 2)
        payload[mode == 2, :8] = ((c4[:, :, 0] << 4) | c4[:, :, 1])[mode == 2]
        payload[mode == 3, :16] = g[mode == 3]
        for m, thr, at in ((1, 3, 4), (2, 15, 8)):
            rows = np.nonzero(mode == m)[0]
            esc = g[rows] >= thr
            order = np.argsort(~esc, axis=1, kind="stable")  # escaped values first, in order
            payload[rows, at:at + 16] = np.where(np.take_along_axis(esc, order, 1),
                                                 np.take_along_axis(g[rows], order, 1), 0)
        hdr = np.zeros((stride, (groups + 3) // 4 * 4), np.uint8)
        hdr[:, :groups] = mode.reshape(stride, groups)
        hdr = hdr.reshape(stride, -1, 4)
        header = (hdr[:, :, 0] | (hdr[:, :, 1] << 2) | (hdr[:, :, 2] << 4) | (hdr[:, :, 3] << 6)).astype(np.uint8)
        keep = np.arange(24)[None, :] < length[:, None]
        body = [payload[k * groups:(k + 1) * groups][keep[k * groups:(k + 1) * groups]] for k in range(stride)]
        for k in range(stride):
            out += [header[k].tobytes(), body[k].tobytes()]
    out.append(bytes(max(stride, 32)))  # padding, then the zero baseline vertex
    return b"".join(out)


def meshopt_encode_index_sequence(indices: np.ndarray) -> bytes:
    """uint32 indices -> an EXT_meshopt_compression INDICES stream (one
    baseline: zig-zag deltas against the previous index)."""
    idx = np.asarray(indices, np.int64).reshape(-1)
    d = np.diff(np.concatenate([[0], idx]))
    d = ((d + (1 << 31)) & 0xFFFFFFFF) - (1 << 31)
    v = (np.where(d >= 0, 2 * d, -2 * d - 1) << 1).astype(np.uint64)  # baseline 0
    out = bytearray([0xD1])
    groups = [(v >> np.uint64(7 * i)) & np.uint64(0x7F) for i in range(5)]
    nbytes = np.maximum(1, (np.floor(np.log2(np.maximum(v, 1).astype(np.float64))) // 7 + 1).astype(np.int64))
    nbytes[v == 0] = 1
    cols = np.stack(groups, 1).astype(np.uint8)
    cols[np.arange(5)[None, :] < (nbytes - 1)[:, None]] |= 0x80
    out += cols[np.arange(5)[None, :] < nbytes[:, None]].tobytes()
    return bytes(out) + bytes(4)


def write_world(path, meshes, world, material: dict | None = None, meshopt: bool = False) -> Path:
    """One glTF mesh per primitive (positions, UVs when present, uint32
    indices, material 0), the world's nodes, first scene and animations, as
    a .glb.  `material` is the glTF material dict (default: white).  With
    `meshopt`, vertex data and indices are EXT_meshopt_compression streams
    (ATTRIBUTES and INDICES)."""
    b = Builder()

    def vertex_accessor(a: np.ndarray) -> int:
        a = np.ascontiguousarray(a, np.float32)
        if not meshopt:
            return b.accessor(a)
        raw = a.reshape(len(a), -1).view(np.uint8)
        view = b.meshopt_view(meshopt_encode_attributes(raw), len(a), raw.shape[1], "ATTRIBUTES",
                              byte_stride=raw.shape[1])
        return b.view_accessor(view, np.float32, len(a), a.shape[1])

    def index_accessor(i: np.ndarray) -> int:
        i = np.ascontiguousarray(i, np.uint32).reshape(-1)
        if not meshopt:
            return b.accessor(i)
        return b.view_accessor(b.meshopt_view(meshopt_encode_index_sequence(i), len(i), 4, "INDICES"),
                               np.uint32, len(i), 1)

    for m in meshes:
        attrs = {"POSITION": vertex_accessor(m.positions)}
        if m.uvs is not None:
            attrs["TEXCOORD_0"] = vertex_accessor(m.uvs)
        b.add("meshes", {"primitives": [{"attributes": attrs, "material": 0, "indices": index_accessor(m.indices)}]})
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
