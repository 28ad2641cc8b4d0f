"""The library's Zstandard decoder (vkgv_zstd_decompress, KTX2
supercompression scheme 2) against real libzstd output: committed frames
(tests/golden/zstd_frames.json, written by make_zstd_vectors.py) and, where
pyarrow is installed, freshly compressed seeded inputs at several levels;
concatenated and skippable frames; the XXH64 content checksum; corrupt,
truncated and oversized inputs return a status, never crash."""
import base64
import ctypes as C
import hashlib
import json
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from vk_gltf_viewer_gb300 import abi, texture

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "zstd_frames.json").read_text())


def _decode(frame: bytes, cap: int):
    src = np.frombuffer(frame, np.uint8) if frame else np.zeros(1, np.uint8)
    out = np.zeros(max(1, cap), np.uint8)
    n = C.c_uint64()
    rc = abi.load().vkgv_zstd_decompress(src.ctypes.data, len(frame), out.ctypes.data, cap, C.byref(n))
    return rc, out[: n.value].tobytes()


def test_golden_frames(built):
    assert len(GOLDEN["cases"]) >= 20
    for c in GOLDEN["cases"]:
        frame = base64.b64decode(c["frame"])
        rc, out = _decode(frame, c["size"])
        assert rc == abi.OK, (c["name"], c["level"])
        assert len(out) == c["size"] and hashlib.sha256(out).hexdigest() == c["sha256"], (c["name"], c["level"])
        if c["size"]:
            assert _decode(frame, c["size"] - 1)[0] == abi.LIMIT_EXCEEDED


def test_fresh_frames_from_libzstd(built):
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(7)
    for trial in range(40):
        kind = trial % 4
        n = int(rng.integers(0, 400000))
        if kind == 0:
            data = rng.integers(0, int(rng.integers(2, 257)), n, dtype=np.uint8).tobytes()
        elif kind == 1:
            words = [bytes(rng.integers(97, 123, int(rng.integers(1, 9)), dtype=np.uint8)) for _ in range(300)]
            data = b" ".join(words[int(i)] for i in rng.integers(0, 300, max(1, n // 6)))
        elif kind == 2:
            data = np.repeat(rng.integers(0, 256, max(1, n // 37), dtype=np.uint8), 37).tobytes()
        else:
            base = rng.integers(0, 256, 4096, dtype=np.uint8)
            data = np.concatenate([np.roll(base, int(s)) for s in rng.integers(0, 4096, max(1, n // 4096))]).tobytes()
        level = int(rng.choice([1, 3, 7, 12, 19, 22, -3]))
        frame = pa.Codec("zstd", compression_level=level).compress(data, asbytes=True)
        rc, out = _decode(frame, len(data))
        assert rc == abi.OK and out == data, (trial, level, len(data))


def test_concatenated_and_skippable_frames(built):
    c = [base64.b64decode(x["frame"]) for x in GOLDEN["cases"][:4]]
    sizes = [x["size"] for x in GOLDEN["cases"][:4]]
    skip = struct.pack("<II", 0x184D2A53, 5) + b"hello"
    rc, out = _decode(c[0] + skip + c[1] + c[2], sum(sizes[:3]))
    assert rc == abi.OK and len(out) == sum(sizes[:3])
    rc0, a = _decode(c[0], sizes[0])
    assert out[: sizes[0]] == a


def test_xxh64_and_content_checksum(built):
    lib = abi.load()
    assert lib.vkgv_xxh64(None, 0) == 0xEF46DB3751D8E999
    # a raw-block frame with the checksum flag: header 0x24 (single segment,
    # checksum), 1-byte content size, one last raw block, 4 checksum bytes
    for payload in (b"", b"x", b"hello zstd", bytes(range(200))):
        buf = np.frombuffer(payload, np.uint8) if payload else np.zeros(1, np.uint8)
        h = lib.vkgv_xxh64(buf.ctypes.data, len(payload))
        block = struct.pack("<I", 1 | (len(payload) << 3))[:3]
        frame = struct.pack("<I", 0xFD2FB528) + bytes([0x24, len(payload)]) + block + payload
        rc, out = _decode(frame + struct.pack("<I", h & 0xFFFFFFFF), len(payload))
        assert rc == abi.OK and out == payload
        rc, _ = _decode(frame + struct.pack("<I", (h ^ 1) & 0xFFFFFFFF), len(payload))
        assert rc == abi.INVALID_ARG


_FUZZ = r"""
import base64, ctypes as C, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from vk_gltf_viewer_gb300 import abi
lib = abi.load()
cases = json.load(open(sys.argv[2]))["cases"]
rng = np.random.default_rng(int(sys.argv[3]))
codes = set()
for it in range(1500):
    c = cases[int(rng.integers(0, len(cases)))]
    f = bytearray(base64.b64decode(c["frame"]))
    if not f:
        continue
    for _ in range(int(rng.integers(1, 4))):
        if not f:
            break
        op = int(rng.integers(0, 3))
        if op == 0:
            f[int(rng.integers(0, len(f)))] = int(rng.integers(0, 256))
        elif op == 1:
            del f[int(rng.integers(0, len(f))):]
        else:
            i = int(rng.integers(0, len(f)))
            f[i] ^= 1 << int(rng.integers(0, 8))
    src = np.frombuffer(bytes(f), np.uint8) if f else np.zeros(1, np.uint8)
    out = np.zeros(c["size"] + 64, np.uint8)
    n = C.c_uint64()
    codes.add(lib.vkgv_zstd_decompress(src.ctypes.data, len(f), out.ctypes.data, out.size, C.byref(n)))
print(sorted(codes))
"""


def test_mutated_frames_return_a_status(built, tmp_path):
    """Seeded mutations (byte changes, bit flips, truncation) of the golden
    frames decode or fail with a status, in a child process so that a crash
    would show as a failure rather than take the test run down."""
    root = Path(__file__).resolve().parent.parent
    script = tmp_path / "fuzz.py"
    script.write_text(_FUZZ)
    res = subprocess.run([sys.executable, str(script), str(root), str(root / "tests" / "golden" / "zstd_frames.json"),
                          "11"], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    codes = set(json.loads(res.stdout.strip().splitlines()[-1]))
    assert codes <= {abi.OK, abi.INVALID_ARG, abi.LIMIT_EXCEEDED}
    assert abi.INVALID_ARG in codes


def test_four_stream_literals_need_six_bytes(built):
    """Four Huffman streams of literals split (n + 3) / 4 to each of the
    first three; a section of 5 literals would give them 6 and the fourth
    a negative count: refused before any stream is decoded."""
    lit_hdr = (2 | (1 << 2) | (5 << 4) | (12 << 14)).to_bytes(3, "little")  # Huffman, 4 streams, 5 literals
    tree = bytes([0x80, 0x10])                       # two symbols of weight 1: 1-bit codes
    jump = (1).to_bytes(2, "little") * 3              # streams of one byte each
    streams = bytes([0x04]) * 4                      # two 1-bit codes, then the end marker
    block = lit_hdr + tree + jump + streams + bytes([0])  # no sequences
    frame = (bytes.fromhex("28b52ffd") + bytes([0x20, 5])
             + (1 | (2 << 1) | (len(block) << 3)).to_bytes(3, "little") + block)
    rc, _ = _decode(frame, 64)
    assert rc == abi.INVALID_ARG


def test_ktx2_zstd_level(built):
    """A KTX2 file whose level is Zstandard-supercompressed (scheme 2) parses
    to the inflated BC1 blocks; a wrong uncompressed length or a corrupt
    frame is refused."""
    from test_texture_decode import _ktx2
    rng = np.random.default_rng(3)
    w, h = 64, 48  # 16 x 12 BC1 blocks of 8 bytes
    blocks = np.tile(rng.integers(0, 256, 64, dtype=np.uint8), 24).tobytes()
    try:
        import pyarrow as pa
        comp = pa.Codec("zstd", compression_level=9).compress(blocks, asbytes=True)
    except ImportError:  # one raw block in a frame is still scheme 2
        comp = struct.pack("<I", 0xFD2FB528) + bytes([0x00]) + struct.pack("<I", 1 | (len(blocks) << 3))[:3] + blocks
    raw_length_at = 96  # the level index's uncompressedByteLength
    data = bytearray(_ktx2(133, w, h, comp, scheme=2))
    struct.pack_into("<Q", data, raw_length_at, len(blocks))
    info, got = texture.parse_ktx2(bytes(data))
    assert info.supercompression == 2 and info.format == abi.BC1 and (info.width, info.height) == (w, h)
    assert got.tobytes() == blocks
    bad = bytearray(data)
    struct.pack_into("<Q", bad, raw_length_at, len(blocks) + 8)
    with pytest.raises(abi.VkgvError):
        texture.parse_ktx2(bytes(bad))
    bad = bytearray(data)
    bad[len(bad) - len(comp)] ^= 0xFF  # the frame's magic number
    with pytest.raises(abi.VkgvError):
        texture.parse_ktx2(bytes(bad))
