"""EXT_meshopt_compression decoding (src/vk_gltf_viewer/assets.cpp:111-166):
the library's decoder (vkgv_meshopt_decode) against the oracle's
restatement and against the data the test encoders were given, for every
mode, stride class and filter; malformed streams fail alike in both; a
glTF asset with compressed views imports exactly like the same asset
without compression."""
import numpy as np
import pytest

from oracle import meshopt as om
from vk_gltf_viewer_gb300 import abi, gltf

from meshopt_util import (encode_attributes, encode_exponential, encode_octahedral, encode_quaternion,
                          encode_sequence, encode_triangles)


def _decode(stream, count, stride, mode, filt=abi.MESHOPT_FILTER_NONE):
    return gltf.meshopt_decode(stream, count, stride, mode, filt).tobytes()


def _ok(stream, count, stride, mode, filt=abi.MESHOPT_FILTER_NONE):
    """Library result or None on failure."""
    try:
        return _decode(stream, count, stride, mode, filt)
    except abi.VkgvError as e:
        assert e.code == abi.INVALID_ARG
        return None


def _vertex_data(rng, count, stride, kind):
    if kind == "random":
        return rng.integers(0, 256, count * stride, dtype=np.uint8).tobytes()
    # smooth: small deltas between neighbours (the codec's target), with outliers
    base = np.cumsum(rng.integers(-3, 4, (count, stride)), 0)
    base[rng.random((count, stride)) < 0.02] += 97
    return (base & 0xFF).astype(np.uint8).tobytes()


@pytest.mark.parametrize("stride", [4, 8, 12, 16, 20, 64, 252, 256])
@pytest.mark.parametrize("count", [0, 1, 15, 16, 17, 100, 257, 700])
def test_attributes_round_trip(built, stride, count):
    rng = np.random.default_rng(stride * 1000 + count)
    for kind in ("smooth", "random"):
        data = _vertex_data(rng, count, stride, kind)
        stream = encode_attributes(data, count, stride, rng)
        assert _decode(stream, count, stride, abi.MESHOPT_ATTRIBUTES) == data
        if count * stride <= 64 * 700:
            assert om.attributes(stream, count, stride) == data


def test_attributes_block_boundaries(built):
    """Counts around the block size min(8192 / stride rounded to 16, 256):
    the delta chain continues from block to block."""
    rng = np.random.default_rng(3)
    for stride in (4, 32, 128, 256):
        block = min((8192 // stride) // 16 * 16, 256)
        for count in (block - 1, block, block + 1, 3 * block + 5):
            data = _vertex_data(rng, count, stride, "smooth")
            stream = encode_attributes(data, count, stride, rng)
            assert _decode(stream, count, stride, abi.MESHOPT_ATTRIBUTES) == data


def test_attributes_large_view_threaded(built):
    """Views of 4 MB and more split their blocks over threads (a pre-scan
    for block starts, chains from zero, then carries): same bytes as the
    data, and a stream cut short or with a byte changed still fails or
    decodes like one thread would (the oracle is too slow at this size, so
    the check is the round trip)."""
    from vk_gltf_viewer_gb300.gltf_export import meshopt_encode_attributes

    rng = np.random.default_rng(8)
    count, stride = 300_001, 16
    base = np.cumsum(rng.integers(-2, 3, (count, stride), dtype=np.int16), 0, dtype=np.int16)
    base[rng.random((count, stride)) < 0.001] += 77
    data = (base & 0xFF).astype(np.uint8)
    stream = meshopt_encode_attributes(data)
    assert _decode(stream, count, stride, abi.MESHOPT_ATTRIBUTES) == data.tobytes()
    with pytest.raises(abi.VkgvError):
        _decode(stream[:-1], count, stride, abi.MESHOPT_ATTRIBUTES)
    with pytest.raises(abi.VkgvError):
        _decode(stream, count + 4096, stride, abi.MESHOPT_ATTRIBUTES)


def _mesh_triangles(rng, n_vert=300, n_tri=600, big=0):
    """Triangles of a vertex-cache-friendly strip, with jumps, repeats and
    (big > 0) indices above 2^16."""
    tris = []
    v = 0
    for i in range(n_tri):
        r = rng.random()
        if r < 0.6:  # a consistently wound strip: neighbours cross their shared edge both ways
            tri = (v, v + 1, v + 2) if i % 2 == 0 else (v + 2, v + 1, v + 3)
            v += 2 if i % 2 else 0
        elif r < 0.8 and tris:
            t = tris[int(rng.integers(0, len(tris)))]
            tri = (t[2], t[1], int(rng.integers(0, n_vert)))
        else:
            tri = tuple(int(x) for x in rng.integers(0, n_vert, 3))
        tris.append(tuple(x + big for x in tri))
    return tris


@pytest.mark.parametrize("version", [0, 1])
@pytest.mark.parametrize("stride", [2, 4])
def test_triangles_round_trip(built, version, stride):
    rng = np.random.default_rng(version * 10 + stride)
    for big in (0, 70000 if stride == 4 else 0):
        tris = _mesh_triangles(rng, big=big)
        stream = encode_triangles(tris, rng, version)
        want = np.asarray(tris, np.uint16 if stride == 2 else np.uint32).tobytes()
        count = 3 * len(tris)
        assert _decode(stream, count, stride, abi.MESHOPT_TRIANGLES) == want
        assert om.triangles(stream, count, stride) == want


def test_triangles_every_code_path(built):
    """Random encodings of one mesh reach every branch: edge + new / FIFO /
    last -+ 1 / explicit third vertex, table codes, 0xFE, 0xFF and restarts."""
    rng = np.random.default_rng(11)
    tris = _mesh_triangles(rng, n_tri=400) + [(0, 1, 2), (5, 0, 1), (0, 1, 2)]
    seen = set()
    for _ in range(6):
        stream = encode_triangles(tris, rng, 1)
        n = len(tris)
        codes = stream[1:1 + n]
        for c in codes:
            seen.add("edge" if c < 0xF0 and (c & 15) == 0 else
                     "edge_fifo" if c < 0xF0 and (c & 15) < 13 else
                     "edge_delta" if c < 0xF0 and (c & 15) < 15 else
                     "edge_explicit" if c < 0xF0 else "table" if c < 0xFE else hex(c))
        assert _decode(stream, 3 * n, 4, abi.MESHOPT_TRIANGLES) == np.asarray(tris, np.uint32).tobytes()
    assert {"edge", "edge_fifo", "edge_delta", "edge_explicit", "table", "0xfe", "0xff"} <= seen


@pytest.mark.parametrize("stride", [2, 4])
def test_sequence_round_trip(built, stride):
    rng = np.random.default_rng(stride)
    top = 60000 if stride == 2 else 1 << 29
    idx = [int(x) for x in rng.integers(0, top, 500)] + list(range(100, 200)) + [0, 0, top - 1]
    stream = encode_sequence(idx, rng)
    want = np.asarray(idx, np.uint16 if stride == 2 else np.uint32).tobytes()
    assert _decode(stream, len(idx), stride, abi.MESHOPT_INDICES) == want
    assert om.sequence(stream, len(idx), stride) == want
    assert _decode(encode_sequence([], rng), 0, stride, abi.MESHOPT_INDICES) == b""


def test_filters_match_oracle_on_every_value(built):
    """Filters over raw values covering the whole integer range (the stream
    only carries them): bit-exact with the oracle's fp32 restatement."""
    rng = np.random.default_rng(5)
    cases = [(4, abi.MESHOPT_FILTER_OCTAHEDRAL, rng.integers(-128, 128, (4096, 4)).astype(np.int8)),
             (8, abi.MESHOPT_FILTER_OCTAHEDRAL, rng.integers(-32768, 32768, (4096, 4)).astype(np.int16)),
             (8, abi.MESHOPT_FILTER_QUATERNION, rng.integers(-32768, 32768, (4096, 4)).astype(np.int16)),
             (8, abi.MESHOPT_FILTER_EXPONENTIAL, rng.integers(0, 1 << 32, (4096, 2), dtype=np.uint64).astype(np.uint32)),
             (12, abi.MESHOPT_FILTER_EXPONENTIAL, rng.integers(0, 1 << 32, (4096, 3), dtype=np.uint64).astype(np.uint32))]
    # also the octahedral corner cases: all zero, the encoded 1.0 alone, extremes
    cases[0][2][:4] = [[0, 0, 0, 0], [0, 0, 127, 5], [127, 0, 0, -1], [-128, -128, -128, -128]]
    cases[1][2][:3] = [[0, 0, 0, 0], [32767, -32768, 1, 9], [0, 0, 4095, 0]]
    for stride, filt, raw in cases:
        data = raw.tobytes()
        count = len(raw)
        stream = encode_attributes(data, count, stride, rng)
        got = _decode(stream, count, stride, abi.MESHOPT_ATTRIBUTES, filt)
        want = om.decode(stream, count, stride, om.ATTRIBUTES, filt)
        if filt == abi.MESHOPT_FILTER_EXPONENTIAL:  # NaN-free: compare bits
            assert np.array_equal(np.frombuffer(got, np.uint32), np.frombuffer(want, np.uint32))
        else:
            assert got == want


def test_filters_reconstruct_encoded_values(built):
    rng = np.random.default_rng(9)
    n = rng.normal(size=(2000, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    for stride, dtype, bits in ((4, np.int8, 8), (8, np.int16, 12), (8, np.int16, 16)):
        w = rng.choice([-1, 1], len(n)) * ((1 << (bits - 1)) - 1)
        raw = encode_octahedral(n, bits, w, dtype)
        stream = encode_attributes(raw.tobytes(), len(n), stride, rng)
        out = np.frombuffer(_decode(stream, len(n), stride, abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_OCTAHEDRAL),
                            dtype).reshape(-1, 4)
        one = float(np.iinfo(dtype).max)
        assert np.abs(out[:, :3] / one - n).max() < 4.0 / (1 << (bits - 1)) + 1.0 / one
        assert np.array_equal(out[:, 3], raw[:, 3])  # w is kept
    q = rng.normal(size=(2000, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    raw = encode_quaternion(q, 16)
    stream = encode_attributes(raw.tobytes(), len(q), 8, rng)
    out = np.frombuffer(_decode(stream, len(q), 8, abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_QUATERNION),
                        np.int16).reshape(-1, 4) / 32767.0
    assert np.minimum(np.abs(out - q).max(1), np.abs(out + q).max(1)).max() < 1e-4
    f = (rng.normal(size=3000) * 10.0 ** rng.integers(-8, 8, 3000)).astype(np.float32)
    f[:3] = [0.0, 1.0, -2.5]
    words = encode_exponential(f, rng)
    stream = encode_attributes(words.tobytes(), len(f) // 3, 12, rng)
    out = np.frombuffer(_decode(stream, len(f) // 3, 12, abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_EXPONENTIAL),
                        np.float32)
    assert np.all(np.abs(out - f) <= np.abs(f) * 2.0 ** -21)
    assert list(out[:3]) == [0.0, 1.0, -2.5]


def test_invalid_arguments(built):
    rng = np.random.default_rng(0)
    good = encode_attributes(bytes(64), 16, 4, rng)
    bad = [(good, 16, 6, abi.MESHOPT_ATTRIBUTES, 0),                       # stride not a multiple of 4
           (good, 16, 260, abi.MESHOPT_ATTRIBUTES, 0),                     # stride above 256
           (good, 16, 4, abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_QUATERNION),  # quaternion needs 8
           (encode_sequence([1, 2, 3], rng), 3, 4, abi.MESHOPT_INDICES, abi.MESHOPT_FILTER_EXPONENTIAL),
           (encode_sequence([1, 2, 3], rng), 3, 8, abi.MESHOPT_INDICES, 0),
           (encode_triangles([(0, 1, 2)], rng), 4, 4, abi.MESHOPT_TRIANGLES, 0),   # count not a multiple of 3
           (good, 16, 4, 7, 0)]
    for stream, count, stride, mode, filt in bad:
        with pytest.raises(abi.VkgvError):
            _decode(stream, count, stride, mode, filt)
    # wrong header, trailing bytes, and declared counts needing more header
    # bytes than the stream holds (up to 64 elements share one header byte
    # per column, whose unused modes read as all-zero groups, so 17 or 40
    # decode this stream too)
    assert len(_decode(good, 40, 4, abi.MESHOPT_ATTRIBUTES)) == 160
    for stream, count in ((b"\xa1" + good[1:], 16), (good + b"\0", 16), (good, 65), (good, 1000)):
        with pytest.raises(abi.VkgvError):
            _decode(stream, count, 4, abi.MESHOPT_ATTRIBUTES)


@pytest.mark.parametrize("mode", ["attributes", "triangles", "sequence"])
def test_malformed_streams_agree_with_oracle(built, mode):
    """Seeded byte flips, truncations and insertions of valid streams: the
    library and the oracle accept the same streams and decode them alike."""
    rng = np.random.default_rng({"attributes": 1, "triangles": 2, "sequence": 3}[mode])
    if mode == "attributes":
        count, stride, m = 90, 12, abi.MESHOPT_ATTRIBUTES
        good = encode_attributes(_vertex_data(rng, count, stride, "smooth"), count, stride, rng)
    elif mode == "triangles":
        tris = _mesh_triangles(rng, n_tri=120)
        count, stride, m = 3 * len(tris), 4, abi.MESHOPT_TRIANGLES
        good = encode_triangles(tris, rng, 1)
    else:
        idx = [int(x) for x in rng.integers(0, 5000, 150)]
        count, stride, m = len(idx), 4, abi.MESHOPT_INDICES
        good = encode_sequence(idx, rng)
    accepted = 0
    for i in range(400):
        data = bytearray(good)
        op = i % 3
        if op == 0:
            for _ in range(int(rng.integers(1, 4))):
                data[int(rng.integers(0, len(data)))] ^= int(rng.integers(1, 256))
        elif op == 1:
            data = data[:int(rng.integers(0, len(data)))]
        else:
            at = int(rng.integers(0, len(data)))
            data[at:at] = bytes(rng.integers(0, 256, int(rng.integers(1, 6)), dtype=np.uint8))
        data = bytes(data)
        want = om.decode(data, count, stride, m)
        got = _ok(data, count, stride, m)
        assert got == want, (i, op)
        accepted += want is not None
    assert 0 < accepted < 400


def _scene_builder(compress: bool, rng):
    """A two-node asset with quantised positions, indices and a rotation +
    translation animation; with `compress`, every buffer view is an
    EXT_meshopt_compression stream (positions ATTRIBUTES, indices
    TRIANGLES, key times EXPONENTIAL, rotations QUATERNION).  The plain
    asset stores the values the filters decode to, so both must import alike."""
    from vk_gltf_viewer_gb300 import scene
    from vk_gltf_viewer_gb300.gltf_export import SHORT, Builder, quantize_i16

    ico = scene.icosphere(3)
    q, s = quantize_i16(ico.positions)
    pos = np.zeros((len(q), 4), np.int16)  # padded to 8 bytes (KHR_mesh_quantization)
    pos[:, :3] = q
    tris = [tuple(int(v) for v in t) for t in ico.indices.reshape(-1, 3)]
    times = np.array([0.0, 0.5, 1.25, 2.0], np.float32)
    t_words = encode_exponential(times, rng)
    quats = rng.normal(size=(4, 4))
    q_raw = encode_quaternion(quats, 16)
    # the values the filters decode to
    times_dec = np.frombuffer(om.exponential(t_words.tobytes(), len(times)), np.float32)
    quats_dec = np.frombuffer(om.quaternion(q_raw.tobytes(), len(quats)), np.int16).reshape(-1, 4)
    moves = np.array([[0, 0, 0], [1, 0, 0], [1, 2, 0], [0, 0, -3]], np.float32)

    b = Builder()
    if compress:
        pv = b.meshopt_view(encode_attributes(pos.tobytes(), len(pos), 8, rng), len(pos), 8, "ATTRIBUTES",
                            byte_stride=8)
        pa = b.view_accessor(pv, np.int16, len(pos), 3, normalized=True)
        iv = b.meshopt_view(encode_triangles(tris, rng, 1), 3 * len(tris), 4, "TRIANGLES")
        ia = b.view_accessor(iv, np.uint32, 3 * len(tris), 1)
        tv = b.meshopt_view(encode_attributes(t_words.tobytes(), len(times), 4, rng), len(times), 4, "ATTRIBUTES",
                            "EXPONENTIAL")
        ta = b.view_accessor(tv, np.float32, len(times), 1)
        rv = b.meshopt_view(encode_attributes(q_raw.tobytes(), len(quats), 8, rng), len(quats), 8, "ATTRIBUTES",
                            "QUATERNION")
        ra = b.view_accessor(rv, np.int16, len(quats), 4, normalized=True)
        mv = b.meshopt_view(encode_attributes(moves.tobytes(), len(moves), 12, rng), len(moves), 12, "ATTRIBUTES")
        ma = b.view_accessor(mv, np.float32, len(moves), 3)
    else:
        pa = b.accessor(pos[:, :3], normalized=True, stride=8)
        ia = b.accessor(np.asarray(tris, np.uint32).reshape(-1))
        ta = b.accessor(times_dec)
        ra = b.accessor(quats_dec, normalized=True)
        ma = b.accessor(moves)
    b.add("meshes", {"primitives": [{"attributes": {"POSITION": pa}, "indices": ia}]})
    b.add("nodes", {"mesh": 0, "children": [1], "scale": [s, s, s]})
    b.add("nodes", {"mesh": 0, "translation": [3, 0, 0]})
    b.gltf["scenes"] = [{"nodes": [0]}]
    b.add("animations", {"samplers": [{"input": ta, "output": ra}, {"input": ta, "output": ma}],
                         "channels": [{"sampler": 0, "target": {"node": 1, "path": "rotation"}},
                                      {"sampler": 1, "target": {"node": 0, "path": "translation"}}]})
    assert b.gltf["accessors"][pa]["componentType"] == SHORT
    return b


@pytest.mark.parametrize("container", ["glb", "gltf"])
def test_gltf_with_compressed_views_imports_like_plain(built, tmp_path, container):
    from oracle import binding as ob

    paths = []
    for compress in (True, False):
        b = _scene_builder(compress, np.random.default_rng(21))
        if compress:
            b.gltf["extensionsRequired"] = ["EXT_meshopt_compression"]
        name = tmp_path / f"{'c' if compress else 'p'}.{container}"
        paths.append(b.write_glb(name) if container == "glb" else b.write_gltf(name))
    (hc, wc), (hp, wp) = (gltf.load(p) for p in paths)
    assert len(hc.meshes) == len(hp.meshes) == 1
    for f in ("positions", "indices"):
        assert np.array_equal(getattr(hc.meshes[0], f), getattr(hp.meshes[0], f))
    assert np.array_equal(hc.draws, hp.draws)
    for t in (0.0, 0.3, 1.0, 1.9, 2.5):
        assert np.array_equal(ob.world_transforms(wc, t), ob.world_transforms(wp, t))


def test_gltf_meshopt_errors(built, tmp_path):
    rng = np.random.default_rng(4)
    b = _scene_builder(True, rng)
    # a corrupt stream: the asset is refused with a message naming the view
    ext = b.gltf["bufferViews"][1]["extensions"]["EXT_meshopt_compression"]
    b.bin[ext["byteOffset"] + 1] ^= 0xFF
    with pytest.raises(abi.VkgvError, match="bufferView 1 does not decode"):
        gltf.load(b.write_glb(tmp_path / "bad.glb"))
    # a plain view reading the fallback buffer (which has no data)
    b = _scene_builder(True, rng)
    b.gltf["bufferViews"].append({"buffer": 1, "byteOffset": 0, "byteLength": 4})
    b.gltf["accessors"][0]["bufferView"] = len(b.gltf["bufferViews"]) - 1
    with pytest.raises(abi.VkgvError, match="without data"):
        gltf.load(b.write_glb(tmp_path / "fallback.glb"))
    b = _scene_builder(True, rng)
    b.gltf["bufferViews"][0]["extensions"]["EXT_meshopt_compression"]["mode"] = "VERTICES"
    with pytest.raises(abi.VkgvError, match="not known"):
        gltf.load(b.write_glb(tmp_path / "mode.glb"))


def test_write_world_meshopt_round_trip(built, tmp_path):
    """The package's writer with meshopt=True (ATTRIBUTES positions and UVs,
    INDICES indices): the asset imports exactly like the uncompressed one."""
    from oracle import binding as ob
    from vk_gltf_viewer_gb300 import scene
    from vk_gltf_viewer_gb300.gltf_export import write_world
    from vk_gltf_viewer_gb300.world import grid_world

    import dataclasses

    mesh = scene.icosphere(3)
    uvs = np.random.default_rng(1).random((len(mesh.positions), 2)).astype(np.float32)
    mesh = dataclasses.replace(mesh, uvs=uvs)
    world = grid_world(1, grid=(3, 2, 2))
    plain = gltf.load(write_world(tmp_path / "p.glb", [mesh], world))
    packed = gltf.load(write_world(tmp_path / "c.glb", [mesh], world, meshopt=True))
    for f in ("positions", "indices", "uvs"):
        assert np.array_equal(getattr(plain[0].meshes[0], f), getattr(packed[0].meshes[0], f))
    assert np.array_equal(plain[0].draws, packed[0].draws)
    assert np.array_equal(ob.world_transforms(plain[1], 0.4), ob.world_transforms(packed[1], 0.4))
    assert (tmp_path / "c.glb").stat().st_size < (tmp_path / "p.glb").stat().st_size
