"""The host decoders (PNG / DEFLATE, JPEG, DDS, KTX2, Zstandard, meshopt
streams, glTF with EXT_meshopt_compression) built from their sources with
AddressSanitizer and UndefinedBehaviorSanitizer into a mutation driver
(tests/sanitize/fuzz_decoders.cpp): seeded mutations of valid inputs must
decode or return a status, with no out-of-bounds access, use after free or
undefined behaviour (any report aborts the driver and fails the test)."""
import base64
import json
import os
import shutil
import struct
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import pytest

from vk_gltf_viewer_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "vk_gltf_viewer_gb300" / "csrc"
SOURCES = ["image.cpp", "jpeg.cpp", "zstd.cpp", "meshopt.cpp", "gltf.cpp", "scene.cpp"]
FLAGS = ["-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
         "-fno-omit-frame-pointer", "-I", str(ROOT / "include"), "-I", str(CSRC)]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not installed")
    out = tmp_path_factory.mktemp("sanitize")
    srcs = [ROOT / "tests" / "sanitize" / "fuzz_decoders.cpp"] + [CSRC / s for s in SOURCES]

    def compile_one(src):
        obj = out / (src.name + ".o")
        return subprocess.run([gxx, *FLAGS, "-c", str(src), "-o", str(obj)], capture_output=True, text=True), obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 1)) as ex:
        results = list(ex.map(compile_one, srcs))
    for res, _ in results:
        if res.returncode != 0:
            if "sanitize" in res.stderr and ("unrecognized" in res.stderr or "cannot find" in res.stderr):
                pytest.skip("g++ has no AddressSanitizer runtime")
            raise AssertionError(res.stderr[-2000:])
    exe = out / "fuzz_decoders"
    res = subprocess.run([gxx, *FLAGS, "-o", str(exe), *[str(o) for _, o in results], "-lpthread"],
                         capture_output=True, text=True)
    if res.returncode != 0:
        if "asan" in res.stderr or "ubsan" in res.stderr:
            pytest.skip("g++ has no sanitizer runtime")
        raise AssertionError(res.stderr[-2000:])
    return exe, out


def _run(driver, kind, seed: bytes, name: str, iterations: int, extra=(), valid=True):
    exe, out = driver
    path = out / name
    path.write_bytes(seed)
    env = {**os.environ, "ASAN_OPTIONS": "detect_leaks=1:abort_on_error=0", "UBSAN_OPTIONS": "print_stacktrace=1"}
    res = subprocess.run([str(exe), kind, str(iterations), str(path), *map(str, extra)], capture_output=True,
                         text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-3000:]
    done, ok = map(int, res.stdout.split())
    assert done == iterations
    assert ok >= 1 if valid else ok == 0  # the unmutated seed decodes (or, for a broken one, fails)
    return ok


def _png():
    from png_util import encode
    from test_texture_decode import _samples

    rng = np.random.default_rng(1)
    out = []
    for ctype, depth, interlace in ((2, 8, False), (6, 16, True), (3, 4, True), (0, 1, False)):
        pal = rng.integers(0, 256, size=(16, 3), dtype=np.uint8) if ctype == 3 else None
        out.append(encode(_samples(rng, 13, 17, ctype, depth, 16), ctype, depth, rng, interlace=interlace,
                          palette=pal))
    return out


def _jpeg():
    from jpeg_util import encode
    from test_jpeg import _image

    seeds = []
    for i, kw in enumerate((dict(sampling=((2, 2), (1, 1), (1, 1)), restart=2),
                            dict(progressive=True, sampling=((2, 1), (1, 1), (1, 1))),
                            dict(mode="gray"))):
        seeds.append(encode(_image(19, 23, i), rng=np.random.default_rng(i), **kw)[0])
    return seeds


@pytest.mark.parametrize("kind", ["png", "jpeg", "dds", "ktx2", "zstd"])
def test_image_decoders_under_sanitizers(driver, kind):
    from test_texture_decode import _dds, _ktx2

    if kind == "png":
        seeds = _png()
    elif kind == "jpeg":
        seeds = _jpeg()
    elif kind == "dds":
        seeds = [_dds(b"DXT1", 11, 6, bytes(range(8)) * 6), _dds(b"DX10", 8, 4, bytes(32), dxgi=98),
                 _dds(b"DX10", 8, 4, bytes(32), dxgi=96), _dds(b"DX10", 3, 5, bytes(60), dxgi=87)]
    elif kind == "ktx2":
        frames = json.loads((ROOT / "tests" / "golden" / "zstd_frames.json").read_text())["cases"]
        bc1 = next(c for c in frames if c["name"] == "bc1_blocks" and c["level"] == 1)
        zk = bytearray(_ktx2(133, 128, 4 * (bc1["size"] // 256), base64.b64decode(bc1["frame"]), scheme=2))
        struct.pack_into("<Q", zk, 96, bc1["size"])
        seeds = [_ktx2(133, 11, 6, bytes(range(8)) * 6), _ktx2(145, 5, 4, bytes(range(32))), bytes(zk)]
    else:
        frames = json.loads((ROOT / "tests" / "golden" / "zstd_frames.json").read_text())["cases"]
        seeds = [base64.b64decode(c["frame"]) for c in frames if c["level"] in (1, 19) and c["size"] > 0][:10]
    for i, seed in enumerate(seeds):
        _run(driver, kind, seed, f"{kind}{i}.bin", 4000 if kind == "jpeg" else 1500)
    if kind == "zstd":
        # four Huffman literal streams for 5 literals, unmutated: a status, no
        # write past the literal buffer
        lit = (2 | (1 << 2) | (5 << 4) | (12 << 14)).to_bytes(3, "little") + bytes([0x80, 0x10])
        block = lit + (1).to_bytes(2, "little") * 3 + bytes([0x04]) * 4 + bytes([0])
        frame = (bytes.fromhex("28b52ffd") + bytes([0x20, 5]) + (1 | (2 << 1) | (len(block) << 3)).to_bytes(3, "little")
                 + block)
        _run(driver, kind, frame, "zstd_bad.bin", 1, valid=False)
    if kind == "jpeg":
        # a Huffman table with three 1-bit codes, unmutated: a status, no
        # write past the lookahead table
        dht = bytes([0xFF, 0xC4, 0x00, 2 + 17 + 3, 0x00, 3] + [0] * 15 + [1, 2, 3])
        _run(driver, kind, seeds[0][:2] + dht + seeds[0][2:], "jpeg_bad.bin", 1, valid=False)


def test_meshopt_streams_under_sanitizers(driver):
    import meshopt_util as mu

    rng = np.random.default_rng(3)
    cases = []
    for stride in (4, 12, 16):
        data = rng.integers(0, 256, 300 * stride, dtype=np.uint8).tobytes()
        cases.append((abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_NONE, 300, stride,
                      mu.encode_attributes(data, 300, stride, rng)))
    tris = rng.integers(0, 200, size=(150, 3))
    for version in (0, 1):
        cases.append((abi.MESHOPT_TRIANGLES, abi.MESHOPT_FILTER_NONE, tris.size, 4,
                      mu.encode_triangles(tris, rng, version=version)))
    seq = rng.integers(0, 1000, 400)
    cases.append((abi.MESHOPT_INDICES, abi.MESHOPT_FILTER_NONE, seq.size, 4, mu.encode_sequence(seq, rng)))
    n = rng.normal(size=(200, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    octa = mu.encode_octahedral(n, 10, np.ones(200), np.int16).astype(np.int16).tobytes()
    cases.append((abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_OCTAHEDRAL, 200, 8, mu.encode_attributes(octa, 200, 8, rng)))
    q = rng.normal(size=(200, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    quat = mu.encode_quaternion(q, 12).astype(np.int16).tobytes()
    cases.append((abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_QUATERNION, 200, 8, mu.encode_attributes(quat, 200, 8, rng)))
    ex = mu.encode_exponential(rng.normal(size=(200, 3)).astype(np.float32), rng).astype(np.uint32).tobytes()
    cases.append((abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_EXPONENTIAL, 200, 12, mu.encode_attributes(ex, 200, 12, rng)))
    for i, (mode, filt, count, stride, stream) in enumerate(cases):
        _run(driver, "meshopt", stream, f"meshopt{i}.bin", 4000, (mode, filt, count, stride))


def test_gltf_loader_under_sanitizers(driver, tmp_path):
    from test_fuzz_inputs import _asset
    from test_meshopt import _scene_builder

    seeds = [(_asset(tmp_path).write_glb(tmp_path / "a.glb"), "a.glb"),
             (_asset(tmp_path).write_gltf(tmp_path / "a.gltf"), "a.gltf"),
             (_scene_builder(True, np.random.default_rng(2)).write_glb(tmp_path / "m.glb"), "m.glb")]
    for path, name in seeds:
        _run(driver, "gltf", Path(path).read_bytes(), name, 300)
