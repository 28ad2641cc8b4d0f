"""Texture decode on the host: the PNG decoder returns exactly the pixels a
PNG encoder was given, for every colour type and bit depth, every filter
type, Adam7 interlacing, tRNS, split IDAT chunks and stored / fixed /
dynamic DEFLATE blocks; corrupt files are refused.  The DDS and KTX2 header
readers, the importer's choice of texture source, and the oracle's BC
decoder on hand-derived blocks."""
import ctypes as C
import struct
import zlib

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, texture

from png_util import encode, expected_rgba

CASES = [  # (colour type, depth)
    (6, 8), (2, 8), (0, 8), (4, 8), (6, 16), (2, 16), (0, 16), (4, 16),
    (0, 1), (0, 2), (0, 4), (3, 1), (3, 2), (3, 4), (3, 8),
]


def _samples(rng, h, w, ctype, depth, palette_size=0):
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = palette_size if ctype == 3 else (1 << depth)
    return rng.integers(0, top, size=(h, w, ch), dtype=np.int64)


@pytest.mark.parametrize("ctype,depth", CASES)
@pytest.mark.parametrize("interlace", [False, True])
def test_png_round_trip(built, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + (7 if interlace else 0))
    h, w = 13, 29  # odd sizes: partial Adam7 passes and bit-packed rows
    palette = trns = None
    if ctype == 3:
        n = min(1 << depth, 200)
        palette = rng.integers(0, 256, size=(n, 3))
        trns = bytes(rng.integers(0, 256, size=n // 2, dtype=np.uint8))
        s = _samples(rng, h, w, ctype, depth, n)
    else:
        s = _samples(rng, h, w, ctype, depth)
        if ctype == 0 and depth == 8:
            trns = struct.pack(">H", int(s[3, 4, 0]))
        if ctype == 2 and depth == 16:
            trns = struct.pack(">HHH", *[int(v) for v in s[5, 6]])
    data = encode(s, ctype, depth, rng, interlace=interlace, palette=palette, trns=trns)
    got = texture.decode_png(data)
    assert np.array_equal(got, expected_rgba(s, ctype, depth, palette, trns))


@pytest.mark.parametrize("level,strategy,split", [(0, zlib.Z_DEFAULT_STRATEGY, 0),
                                                  (1, zlib.Z_FIXED, 0),
                                                  (9, zlib.Z_DEFAULT_STRATEGY, 97),
                                                  (6, zlib.Z_HUFFMAN_ONLY, 5),
                                                  (6, zlib.Z_RLE, 0)])
def test_png_deflate_block_kinds(built, level, strategy, split):
    """Stored, fixed-Huffman and dynamic-Huffman blocks, long matches
    (a repetitive image) and IDAT data split over many chunks."""
    rng = np.random.default_rng(level + 10 * split)
    h, w = 64, 96
    base = rng.integers(0, 256, size=(8, w, 4))
    s = np.concatenate([base] * (h // 8))  # repeats: back-references
    s[::7, ::5] = rng.integers(0, 256, size=s[::7, ::5].shape)
    data = encode(s, 6, 8, rng, level=level, strategy=strategy, idat_split=split)
    assert np.array_equal(texture.decode_png(data), s.astype(np.uint8))


def test_png_errors(built):
    rng = np.random.default_rng(1)
    good = encode(_samples(rng, 8, 8, 6, 8), 6, 8, rng)
    bad_crc = bytearray(good)
    bad_crc[20] ^= 0xFF  # inside IHDR: its CRC no longer matches
    cut = good[:len(good) - 30]
    for data, match in [(bytes(bad_crc), "CRC"), (b"not a png at all", "not a PNG"), (cut, None)]:
        with pytest.raises(abi.VkgvError, match=match):
            texture.decode_png(data)


def _dds(fourcc: bytes, w: int, h: int, payload: bytes, dxgi: int | None = None) -> bytes:
    hdr = bytearray(128)
    hdr[0:4] = b"DDS "
    struct.pack_into("<IIIII", hdr, 4, 124, 0x1007, h, w, 0)
    struct.pack_into("<I", hdr, 28, 1)
    struct.pack_into("<II", hdr, 76, 32, 0x4)
    hdr[84:88] = fourcc
    out = bytes(hdr)
    if dxgi is not None:
        out += struct.pack("<IIIII", dxgi, 3, 0, 1, 0)
    return out + payload


def test_dds_headers(built):
    blocks = bytes(range(8)) * 6  # 3 x 2 blocks of 8 bytes
    info, got = texture.parse_dds(_dds(b"DXT1", 11, 6, blocks))
    assert (info.width, info.height, info.format, info.srgb) == (11, 6, abi.BC1, 0)
    assert got.tobytes() == blocks
    info, _ = texture.parse_dds(_dds(b"DXT5", 4, 4, bytes(16)))
    assert info.format == abi.BC3
    info, _ = texture.parse_dds(_dds(b"ATI2", 4, 4, bytes(16)))
    assert info.format == abi.BC5
    info, _ = texture.parse_dds(_dds(b"DX10", 8, 4, bytes(32), dxgi=72))  # BC1_UNORM_SRGB
    assert (info.format, info.srgb, info.data_offset) == (abi.BC1, 1, 148)
    with pytest.raises(abi.VkgvError):
        texture.parse_dds(_dds(b"DXT1", 16, 16, bytes(8)))  # too little data
    with pytest.raises(abi.VkgvError):
        texture.parse_dds(_dds(b"DX10", 4, 4, bytes(16), dxgi=98))  # BC7 is not decoded


def _rgba(r, g, b, a=255):
    return r | (g << 8) | (b << 16) | (a << 24)


def test_oracle_bc_known_answers(built):
    # BC1, four colours: red 0xF800 and blue 0x001F; indices 0,1,2,3 in row 0
    blk = struct.pack("<HHI", 0xF800, 0x001F, 0b11100100)
    out = ob.decode_bc(abi.BC1, np.frombuffer(blk, np.uint8), 4, 4)
    assert list(out[0]) == [_rgba(255, 0, 0), _rgba(0, 0, 255), _rgba(170, 0, 85), _rgba(85, 0, 170)]
    assert out[1, 0] == _rgba(255, 0, 0)
    # BC1, three colours (c0 <= c1): the half-way colour and transparent black
    blk = struct.pack("<HHI", 0x001F, 0xF800, 0b11100100)
    out = ob.decode_bc(abi.BC1, np.frombuffer(blk, np.uint8), 4, 4)
    assert list(out[0]) == [_rgba(0, 0, 255), _rgba(255, 0, 0), _rgba(128, 0, 128), 0]
    # BC4 with a0 > a1: codes 0..7 for texels 0..7
    codes = sum(c << (3 * i) for i, c in enumerate(range(8)))
    blk = bytes([200, 60]) + codes.to_bytes(6, "little")
    out = ob.decode_bc(abi.BC4, np.frombuffer(blk, np.uint8), 4, 4)
    want = [200, 60] + [((7 - j) * 200 + j * 60 + 3) // 7 for j in range(1, 7)]
    assert [int(v) & 255 for v in out.reshape(-1)[:8]] == want
    # a0 <= a1: four steps, then 0 and 255
    blk = bytes([40, 240]) + codes.to_bytes(6, "little")
    out = ob.decode_bc(abi.BC4, np.frombuffer(blk, np.uint8), 4, 4)
    want = [40, 240] + [((5 - j) * 40 + j * 240 + 2) // 5 for j in range(1, 5)] + [0, 255]
    assert [int(v) & 255 for v in out.reshape(-1)[:8]] == want
    # BC2: explicit alpha nibbles, colours always in four-colour mode
    alpha = bytes([0x10, 0xF5] + [0] * 6)
    blk = alpha + struct.pack("<HHI", 0x001F, 0xF800, 0b10)
    out = ob.decode_bc(abi.BC2, np.frombuffer(blk, np.uint8), 4, 4)
    assert out[0, 0] == _rgba(85, 0, 170, 0) and out[0, 1] == _rgba(0, 0, 255, 17)
    assert out[0, 2] >> 24 == 5 * 17 and out[0, 3] >> 24 == 255


def _ktx2(vk_format: int, w: int, h: int, payload: bytes, scheme: int = 0, faces: int = 1, layers: int = 0,
          depth: int = 0) -> bytes:
    """A KTX 2.0 file with one level (no DFD or key/value data)."""
    ident = bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x32, 0x30, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    header = struct.pack("<9I", vk_format, 1, w, h, depth, layers, faces, 1, scheme)
    index = struct.pack("<4I2Q", 0, 0, 0, 0, 0, 0)
    offset = 12 + len(header) + len(index) + 24
    offset += -offset % 16
    level = struct.pack("<3Q", offset, len(payload), len(payload))
    head = ident + header + index + level
    return head + bytes(offset - len(head)) + payload


def test_ktx2_headers(built):
    blocks = bytes(range(8)) * 6  # 3 x 2 blocks of 8 bytes
    for vk, fmt, srgb in ((133, abi.BC1, 0), (131, abi.BC1_OPAQUE, 0), (132, abi.BC1_OPAQUE, 1), (139, abi.BC4, 0)):
        info, got = texture.parse_ktx2(_ktx2(vk, 11, 6, blocks))
        assert (info.width, info.height, info.format, info.srgb) == (11, 6, fmt, srgb)
        assert got.tobytes() == blocks
    info, _ = texture.parse_ktx2(_ktx2(138, 8, 4, bytes(32)))
    assert (info.format, info.srgb) == (abi.BC3, 1)
    rgba = bytes(range(256)) * 3
    info, got = texture.parse_ktx2(_ktx2(43, 16, 12, rgba))
    assert (info.format, info.srgb, info.data_size) == (abi.RGBA8, 1, 768)
    assert np.array_equal(texture.load_image(_ktx2(37, 16, 12, rgba), abi.IMAGE_KTX2).reshape(-1),
                          np.frombuffer(rgba, np.uint8))
    bad = [_ktx2(0, 4, 4, bytes(64)),                  # BasisU (vkFormat undefined)
           _ktx2(133, 4, 4, bytes(8), scheme=1),       # BasisLZ supercompression
           _ktx2(133, 4, 4, bytes(48), faces=6),       # cube map
           _ktx2(140, 4, 4, bytes(8)),                 # BC4 SNORM
           _ktx2(146, 4, 4, bytes(16)),                # BC7
           _ktx2(133, 16, 16, bytes(8)),               # too little data
           b"DDS " + bytes(200)]
    for data in bad:
        with pytest.raises(abi.VkgvError):
            texture.parse_ktx2(data)


def test_oracle_bc1_opaque_known_answer(built):
    """Vulkan's BC1_RGB formats: the three-colour mode's fourth entry is
    opaque black instead of transparent black."""
    blk = struct.pack("<HHI", 0x001F, 0xF800, 0b11100100)
    out = ob.decode_bc(abi.BC1_OPAQUE, np.frombuffer(blk, np.uint8), 4, 4)
    assert list(out[0]) == [_rgba(0, 0, 255), _rgba(255, 0, 0), _rgba(128, 0, 128), _rgba(0, 0, 0, 255)]


def test_gltf_texture_sources(built, tmp_path):
    """MSFT_texture_dds takes precedence; a KHR_texture_basisu (KTX2) source
    is used only when the texture has no base source; the extensions the
    reference enables may be required."""
    from test_gltf_import import make_asset

    b, _ = make_asset()
    ktx = _ktx2(133, 4, 4, bytes(8))
    dds = _dds(b"DXT1", 4, 4, bytes(8))
    png = encode(np.zeros((2, 2, 4), np.int64), 6, 8, np.random.default_rng(0))
    views = [b._view(x) for x in (png, ktx, dds)]
    b.gltf["images"] = [{"bufferView": v, "mimeType": m} for v, m in
                        zip(views, ["image/png", "image/ktx2", "image/vnd-ms.dds"])]
    b.gltf["textures"] = [{"source": 0, "extensions": {"KHR_texture_basisu": {"source": 1}}},
                          {"extensions": {"KHR_texture_basisu": {"source": 1}}},
                          {"source": 0, "extensions": {"MSFT_texture_dds": {"source": 2}}}]
    b.gltf["extensionsRequired"] = ["KHR_texture_basisu", "MSFT_texture_dds", "KHR_lights_punctual"]
    path = b.write_glb(tmp_path / "t.glb")
    lib = abi.load()
    h = C.c_void_p()
    err = C.create_string_buffer(256)
    assert lib.vkgv_gltf_load(str(path).encode(), abi.GLTF_IMAGES, C.byref(h), err, len(err)) == abi.OK, err.value
    try:
        kinds = []
        for t in range(3):
            gi = abi.GltfImage()
            abi.check(lib.vkgv_gltf_get_texture_image(h, t, C.byref(gi)))
            kinds.append(gi.kind)
    finally:
        lib.vkgv_gltf_free(h)
    assert kinds == [abi.IMAGE_PNG, abi.IMAGE_KTX2, abi.IMAGE_DDS]
