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
    info, _ = texture.parse_dds(_dds(b"DX10", 8, 4, bytes(32), dxgi=98))  # BC7_UNORM
    assert (info.format, info.srgb, info.data_size) == (abi.BC7, 0, 32)
    info, _ = texture.parse_dds(_dds(b"DX10", 8, 4, bytes(32), dxgi=99))  # BC7_UNORM_SRGB
    assert (info.format, info.srgb) == (abi.BC7, 1)
    info, _ = texture.parse_dds(_dds(b"DX10", 8, 4, bytes(32), dxgi=95))  # BC6H_UF16
    assert (info.format, info.srgb, info.data_size) == (abi.BC6H_UF16, 0, 32)
    info, _ = texture.parse_dds(_dds(b"DX10", 5, 5, bytes(64), dxgi=96))  # BC6H_SF16
    assert (info.format, info.data_size) == (abi.BC6H_SF16, 64)
    with pytest.raises(abi.VkgvError):
        texture.parse_dds(_dds(b"DX10", 4, 4, bytes(16), dxgi=94))  # BC6H_TYPELESS: no sign to read it with


def _dds_rgb(w: int, h: int, pf_flags: int, masks, payload: bytes) -> bytes:
    """A legacy DDS header with an uncompressed DDPF_RGB pixel format."""
    hdr = bytearray(128)
    hdr[0:4] = b"DDS "
    struct.pack_into("<IIIII", hdr, 4, 124, 0x100F, h, w, w * 4)
    struct.pack_into("<I", hdr, 28, 1)
    struct.pack_into("<IIIIIIII", hdr, 76, 32, pf_flags, 0, 32, *masks)
    return bytes(hdr) + payload


def test_uncompressed_dds(built):
    """32-bit DDS texels decode on the host: DX10 R8G8B8A8 / B8G8R8A8 /
    B8G8R8X8, and legacy RGB pixel formats with RGBA or BGRA byte masks, with
    or without an alpha channel (without one, alpha reads 255)."""
    rng = np.random.default_rng(9)
    px = rng.integers(0, 256, size=(5, 7, 4), dtype=np.uint8)
    bgra = px[..., [2, 1, 0, 3]].copy()
    opaque = px.copy()
    opaque[..., 3] = 255
    rgba_masks = (0x000000FF, 0x0000FF00, 0x00FF0000, 0xFF000000)
    bgra_masks = (0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000)
    cases = [(_dds(b"DX10", 7, 5, px.tobytes(), dxgi=28), abi.RGBA8, 0, px),
             (_dds(b"DX10", 7, 5, px.tobytes(), dxgi=29), abi.RGBA8, 1, px),
             (_dds(b"DX10", 7, 5, bgra.tobytes(), dxgi=87), abi.BGRA8, 0, px),
             (_dds(b"DX10", 7, 5, bgra.tobytes(), dxgi=91), abi.BGRA8, 1, px),
             (_dds(b"DX10", 7, 5, bgra.tobytes(), dxgi=88), abi.BGRX8, 0, opaque),
             (_dds_rgb(7, 5, 0x41, rgba_masks, px.tobytes()), abi.RGBA8, 0, px),
             (_dds_rgb(7, 5, 0x41, bgra_masks, bgra.tobytes()), abi.BGRA8, 0, px),
             (_dds_rgb(7, 5, 0x40, rgba_masks, px.tobytes()), abi.RGBX8, 0, opaque),
             (_dds_rgb(7, 5, 0x40, bgra_masks, bgra.tobytes()), abi.BGRX8, 0, opaque)]
    for data, fmt, srgb, exp in cases:
        info, _ = texture.parse_dds(data)
        assert (info.width, info.height, info.format, info.srgb, info.data_size) == (7, 5, fmt, srgb, 140)
        assert np.array_equal(texture.load_image(data, abi.IMAGE_DDS), exp)  # no renderer needed
    bad = [_dds(b"DX10", 7, 5, px.tobytes()[:-1], dxgi=28),                 # one byte short
           _dds_rgb(7, 5, 0x41, (0xF800, 0x07E0, 0x001F, 0), px.tobytes()),  # 565 masks
           _dds_rgb(7, 5, 0x1, rgba_masks, px.tobytes()),                     # neither RGB nor FourCC
           _dds(b"DX10", 1 << 21, 4, px.tobytes(), dxgi=28)]                 # absurd width
    for data in bad:
        with pytest.raises(abi.VkgvError):
            texture.parse_dds(data)


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
    for vk, srgb in ((145, 0), (146, 1)):
        info, got = texture.parse_ktx2(_ktx2(vk, 5, 4, bytes(range(32))))
        assert (info.format, info.srgb, got.tobytes()) == (abi.BC7, srgb, bytes(range(32)))
    for vk, fmt in ((143, abi.BC6H_UF16), (144, abi.BC6H_SF16)):
        info, got = texture.parse_ktx2(_ktx2(vk, 5, 4, bytes(range(32))))
        assert (info.format, info.srgb, got.tobytes()) == (fmt, 0, bytes(range(32)))
    rgba = bytes(range(256)) * 3
    info, got = texture.parse_ktx2(_ktx2(43, 16, 12, rgba))
    assert (info.format, info.srgb, info.data_size) == (abi.RGBA8, 1, 768)
    assert np.array_equal(texture.load_image(_ktx2(37, 16, 12, rgba), abi.IMAGE_KTX2).reshape(-1),
                          np.frombuffer(rgba, np.uint8))
    bad = [_ktx2(0, 4, 4, bytes(64)),                  # BasisU (vkFormat undefined)
           _ktx2(133, 4, 4, bytes(8), scheme=1),       # BasisLZ supercompression
           _ktx2(133, 4, 4, bytes(48), faces=6),       # cube map
           _ktx2(140, 4, 4, bytes(8)),                 # BC4 SNORM
           _ktx2(133, 16, 16, bytes(8)),               # too little data
           b"DDS " + bytes(200)]
    for data in bad:
        with pytest.raises(abi.VkgvError):
            texture.parse_ktx2(data)


def _bc6h_kat_block(v: int) -> np.ndarray:
    return np.frombuffer(v.to_bytes(16, "little"), np.uint8)


def test_oracle_bc6h_known_answers(built):
    """BC6H answers derived by hand from the format's steps (not from the
    oracle).  Mode 0x03: one region, 10-bit untransformed end points
    (R, G, B) = (1023, 0, 512) and (0, 1023, 512), texels 0, 1, 2 at indices
    0, 15, 7 (weights 0, 64, 30).  Unsigned: 1023 -> 0xFFFF, 512 ->
    ((512 << 16) + 0x8000) >> 10 = 32800, texel 2 R = (34 * 65535 + 32) >> 6
    = 34815, G = (30 * 65535 + 32) >> 6 = 30720; binary16 = v * 31 >> 6.
    Signed: 1023 is -1 -> -(((1 << 15) + 0x4000) >> 9) = -96, 512 is -512 ->
    -0x7FFF; texel 2 R = floor(-3232 / 64) = -51 -> -(51 * 31 >> 5) = -49,
    G = floor(-2848 / 64) = -45 -> -43."""
    v = 0x03 | 1023 << 5 | 0 << 15 | 512 << 25 | 0 << 35 | 1023 << 45 | 512 << 55 | 15 << 68 | 7 << 72
    blk = _bc6h_kat_block(v)
    uf = ob.decode_bc6h(blk, 4, 4, False).reshape(16, 3)
    assert uf[:3].tolist() == [[0x7BFF, 0, 0x3E0F], [0, 0x7BFF, 0x3E0F], [0x41DF, 0x3A20, 0x3E0F]]
    assert uf[3:].tolist() == [[0x7BFF, 0, 0x3E0F]] * 13
    sf = ob.decode_bc6h(blk, 4, 4, True).reshape(16, 3)
    assert sf[:3].tolist() == [[0x805D, 0, 0xFBFF], [0, 0x805D, 0xFBFF], [0x8031, 0x802B, 0xFBFF]]
    # Mode 0x0F stores the base end point's bits 10-15 reversed: block bit
    # 39 is R[15], so R = 0x8000 (unquantised as is at 16 bits), binary16
    # 0x8000 * 31 >> 6 = 0x3E00 (1.5) on every texel (index 0)
    uf = ob.decode_bc6h(_bc6h_kat_block(0x0F | 1 << 39), 4, 4, False).reshape(16, 3)
    assert uf.tolist() == [[0x3E00, 0, 0]] * 16
    # a reserved mode decodes to 0; an interpolated -0 is +0
    assert not ob.decode_bc6h(_bc6h_kat_block(0x13 | 0xFFFF << 20), 4, 4, True).any()


def test_oracle_bc6h_matches_texture_unit_golden(built):
    """The BC6H oracle against the GPU texture unit's decodes of seeded
    blocks of every mode field value, committed by
    tests/golden/make_bc6h_golden.py: identical binary16 texels, UF16 and
    SF16."""
    import base64
    import json
    from pathlib import Path

    g = json.loads((Path(__file__).resolve().parent / "golden" / "bc6h_texture_unit.json").read_text())
    w, h = g["width"], g["height"]
    blocks = np.frombuffer(base64.b64decode(g["blocks"]), np.uint8)
    for key, signed in (("uf16", False), ("sf16", True)):
        exp = np.frombuffer(base64.b64decode(g[key]), np.uint16).reshape(h, w, 3)
        assert np.array_equal(ob.decode_bc6h(blocks, w, h, signed), exp), key


def test_oracle_bc1_opaque_known_answer(built):
    """Vulkan's BC1_RGB formats: the three-colour mode's fourth entry is
    opaque black instead of transparent black."""
    blk = struct.pack("<HHI", 0x001F, 0xF800, 0b11100100)
    out = ob.decode_bc(abi.BC1_OPAQUE, np.frombuffer(blk, np.uint8), 4, 4)
    assert list(out[0]) == [_rgba(0, 0, 255), _rgba(255, 0, 0), _rgba(128, 0, 128), _rgba(0, 0, 0, 255)]


# BC7 mode fields: subsets, partition bits, rotation bits, index-selection
# bits, colour bits, alpha bits, p-bit per endpoint, p-bit per subset, index
# bits, second index bits (the format's mode table)
BC7_MODES = {0: (3, 4, 0, 0, 4, 0, 1, 0, 3, 0), 1: (2, 6, 0, 0, 6, 0, 0, 1, 3, 0), 2: (3, 6, 0, 0, 5, 0, 0, 0, 2, 0),
             3: (2, 6, 0, 0, 7, 0, 1, 0, 2, 0), 4: (1, 0, 2, 1, 5, 6, 0, 0, 2, 3), 5: (1, 0, 2, 0, 7, 8, 0, 0, 2, 2),
             6: (1, 0, 0, 0, 7, 7, 1, 0, 4, 0), 7: (2, 6, 0, 0, 5, 5, 1, 0, 2, 0)}
BC7_WEIGHTS = {2: [0, 21, 43, 64], 3: [0, 9, 18, 27, 37, 46, 55, 64],
               4: [0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64]}


def bc7_block(mode, ep, pbits=(), idx=(), idx2=(), part=0, rot=0, isel=0, anchors=(0,)):
    """Packs one BC7 block from its fields, least significant bit first:
    ep[subset][endpoint] = (r, g, b, a) at the mode's stored precision;
    `anchors` are the texels whose first index is one bit shorter."""
    ns, pb, rb, sb, cb, ab, epb, spb, ib, ib2 = BC7_MODES[mode]
    fields = [(1 << mode, mode + 1), (part, pb), (rot, rb), (isel, sb)]
    fields += [(ep[s][e][c], cb) for c in range(3) for s in range(ns) for e in range(2)]
    fields += [(ep[s][e][3], ab) for s in range(ns) for e in range(2)] if ab else []
    assert len(pbits) == (2 * ns if epb else ns if spb else 0)
    fields += [(p, 1) for p in pbits]
    fields += [(v, ib - (i in anchors)) for i, v in enumerate(idx)]
    fields += [(v, ib2 - (i == 0)) for i, v in enumerate(idx2)]
    word, at = 0, 0
    for v, n in fields:
        assert 0 <= v < (1 << n) or n == 0 and v == 0
        word |= v << at
        at += n
    assert at == 128
    return word.to_bytes(16, "little")


def _bc7_texel(e0, e1, bits, w):
    """One channel: endpoints of `bits` bits (p-bit included) expanded to 8 by
    replicating their top bits, then interpolated with weight w of 64."""
    x0, x1 = e0 << (8 - bits), e1 << (8 - bits)
    x0, x1 = x0 | (x0 >> bits), x1 | (x1 >> bits)
    return ((64 - w) * x0 + w * x1 + 32) >> 6


def test_oracle_bc7_known_answers(built):
    rng = np.random.default_rng(7)

    def decode(blk):
        return ob.decode_bc(abi.BC7, np.frombuffer(blk, np.uint8), 4, 4).reshape(-1)

    def texels(out):
        return [[(int(t) >> (8 * c)) & 255 for c in range(4)] for t in out]

    # mode 6: one subset, RGBA 7 bits + a p-bit per end point, 4-bit indices
    ep = [[(10, 20, 30, 127), (100, 50, 0, 0)]]
    idx = [int(v) for v in rng.integers(0, 16, 16)]
    idx[0] &= 7
    got = texels(decode(bc7_block(6, ep, pbits=(1, 0), idx=idx)))
    for i in range(16):
        want = [_bc7_texel((ep[0][0][c] << 1) | 1, ep[0][1][c] << 1, 8, BC7_WEIGHTS[4][idx[i]]) for c in range(4)]
        assert got[i] == want, i
    # mode 5 with rotation 1: alpha swaps with red after interpolation
    ep = [[(127, 3, 64, 200), (0, 120, 64, 17)]]
    idx, idx2 = [int(v) for v in rng.integers(0, 4, 16)], [int(v) for v in rng.integers(0, 4, 16)]
    idx[0] &= 1
    idx2[0] &= 1
    got = texels(decode(bc7_block(5, ep, idx=idx, idx2=idx2, rot=1)))
    for i in range(16):
        rgb = [_bc7_texel(ep[0][0][c], ep[0][1][c], 7, BC7_WEIGHTS[2][idx[i]]) for c in range(3)]
        a = _bc7_texel(ep[0][0][3], ep[0][1][3], 8, BC7_WEIGHTS[2][idx2[i]])
        assert got[i] == [a, rgb[1], rgb[2], rgb[0]], i
    # mode 4: the index-selection bit gives colour the 3-bit indices; rotation 3 swaps blue
    ep = [[(31, 0, 9, 63), (2, 17, 30, 5)]]
    idx, idx2 = [int(v) for v in rng.integers(0, 4, 16)], [int(v) for v in rng.integers(0, 8, 16)]
    idx[0] &= 1
    idx2[0] &= 3
    for isel in (0, 1):
        got = texels(decode(bc7_block(4, ep, idx=idx, idx2=idx2, isel=isel, rot=3)))
        for i in range(16):
            cw = BC7_WEIGHTS[3][idx2[i]] if isel else BC7_WEIGHTS[2][idx[i]]
            aw = BC7_WEIGHTS[2][idx[i]] if isel else BC7_WEIGHTS[3][idx2[i]]
            rgb = [_bc7_texel(ep[0][0][c], ep[0][1][c], 5, cw) for c in range(3)]
            a = _bc7_texel(ep[0][0][3], ep[0][1][3], 6, aw)
            assert got[i] == [rgb[0], rgb[1], a, rgb[2]], (isel, i)
    # mode 1, two-subset partition 13: rows 0-1 subset 0, rows 2-3 subset 1
    # (anchor texel 15); one p-bit per subset, RGB only
    ep = [[(63, 0, 10, 0), (0, 63, 20, 0)], [(5, 6, 7, 0), (40, 41, 42, 0)]]
    idx = [int(v) for v in rng.integers(0, 8, 16)]
    idx[0] &= 3
    idx[15] &= 3
    got = texels(decode(bc7_block(1, ep, pbits=(1, 0), idx=idx, part=13, anchors=(0, 15))))
    for i in range(16):
        s, p = (0, 1) if i < 8 else (1, 0)
        want = [_bc7_texel((ep[s][0][c] << 1) | p, (ep[s][1][c] << 1) | p, 7, BC7_WEIGHTS[3][idx[i]])
                for c in range(3)]
        assert got[i] == want + [255], i
    # mode 0, three-subset partition 0: columns 0-1 of rows 0-1 and column 0
    # of row 2 subset 0, columns 2-3 of rows 0-2 subset 1, the rest subset 2;
    # anchors at texels 0, 3 and 15
    subset = [0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 2, 1, 2, 2, 2, 2]
    ep = [[(1, 2, 3, 0), (15, 14, 13, 0)], [(4, 4, 4, 0), (9, 0, 15, 0)], [(0, 0, 0, 0), (15, 15, 15, 0)]]
    pbits = (1, 0, 0, 1, 1, 1)
    idx = [int(v) for v in rng.integers(0, 8, 16)]
    for a in (0, 3, 15):
        idx[a] &= 3
    got = texels(decode(bc7_block(0, ep, pbits=pbits, idx=idx, part=0, anchors=(0, 3, 15))))
    for i in range(16):
        s = subset[i]
        p0, p1 = pbits[2 * s], pbits[2 * s + 1]
        want = [_bc7_texel((ep[s][0][c] << 1) | p0, (ep[s][1][c] << 1) | p1, 5, BC7_WEIGHTS[3][idx[i]])
                for c in range(3)]
        assert got[i] == want + [255], i
    # a reserved mode (first byte 0) decodes to transparent black
    assert not decode(bytes(16)).any()
    assert not decode(bytes([0]) + bytes(range(1, 16))).any()


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
