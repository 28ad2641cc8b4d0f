"""Block-compressed textures decoded on the device (k_decode_bc,
k_decode_bc7, k_decode_bc6h) are bit-identical to the oracle's decoder for
BC1-BC5, BC7 and BC6H at block-aligned and ragged sizes, and the BC6H and
BC7 oracles to the GPU texture unit's own decode; JPEG pixels (k_jpeg_idct, k_jpeg_color) are bit-identical to the
oracle's from the same coefficients; and a glTF asset whose base colour comes from an embedded DDS
(MSFT_texture_dds) and PNG renders, textured, like the oracle frame of the
same decoded images."""
import dataclasses

import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, gltf, scene, texture
from vk_gltf_viewer_gb300.gltf_export import Builder
from vk_gltf_viewer_gb300.renderer import ViewBuffers
from vk_gltf_viewer_gb300.world import grid_world

from gpu_util import oracle_flags, rgba_close, small_grid, u32, u64
from png_util import encode
from test_texture_decode import _dds

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [abi.BC1, abi.BC2, abi.BC3, abi.BC4, abi.BC5, abi.BC1_OPAQUE])
@pytest.mark.parametrize("size", [(4, 4), (37, 21), (256, 128), (3, 5)])
def test_bc_decode_matches_oracle(renderer, fmt, size):
    w, h = size
    rng = np.random.default_rng(fmt * 1000 + w)
    bsize = 8 if fmt in (abi.BC1, abi.BC4, abi.BC1_OPAQUE) else 16
    blocks = rng.integers(0, 256, size=((w + 3) // 4) * ((h + 3) // 4) * bsize, dtype=np.uint8)
    if fmt in (abi.BC1, abi.BC4, abi.BC1_OPAQUE):  # both orders of the two end points
        blocks[::16] = np.minimum(blocks[::16], 127)
    got = texture.decode_bc(renderer, fmt, blocks, w, h)
    torch.cuda.synchronize()
    exp = ob.decode_bc(fmt, blocks, w, h)
    assert np.array_equal(got.cpu().numpy().reshape(h, w, 4).view(np.uint32)[..., 0], exp)


def _bc7_blocks(rng, n: int, reserved: bool = True) -> np.ndarray:
    """n random BC7 blocks, every mode equally often (and, with `reserved`,
    blocks whose first byte is 0): any 128 bits after the mode bits are a
    valid block."""
    blocks = rng.integers(0, 256, size=(n, 16), dtype=np.uint8)
    modes = np.arange(n) % (9 if reserved else 8)
    rng.shuffle(modes)
    for mode in range(8):
        rows = modes == mode
        low = (1 << (mode + 1)) - 1
        blocks[rows, 0] = (blocks[rows, 0] & ~np.uint8(low)) | np.uint8(1 << mode)
    blocks[modes == 8, 0] = 0
    return blocks.reshape(-1)


@pytest.mark.parametrize("size", [(4, 4), (37, 21), (256, 128), (3, 5), (1024, 1000)])
def test_bc7_decode_matches_oracle(renderer, size):
    w, h = size
    rng = np.random.default_rng(w * 7 + h)
    blocks = _bc7_blocks(rng, ((w + 3) // 4) * ((h + 3) // 4))
    got = texture.decode_bc(renderer, abi.BC7, blocks, w, h)
    torch.cuda.synchronize()
    exp = ob.decode_bc(abi.BC7, blocks, w, h)
    assert np.array_equal(got.cpu().numpy().reshape(h, w, 4).view(np.uint32)[..., 0], exp)


@pytest.fixture(scope="module")
def texture_unit(tmp_path_factory):
    """Runs tests/bc_hw.cu (built here with nvcc): blocks -> RGBA8 texels
    decoded by the GPU's texture unit from a block-compressed CUDA array."""
    import shutil
    import subprocess
    from pathlib import Path

    tmp = tmp_path_factory.mktemp("bc_hw")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp / "bc_hw"
    src = Path(__file__).with_name("bc_hw.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", str(exe), str(src)],
                   check=True, capture_output=True, timeout=300)

    def decode(fmt: int, blocks: np.ndarray, w: int, h: int) -> np.ndarray:
        """(h, w) uint32 RGBA8, or for BC6H (h, w, 4) float32 RGBA."""
        (tmp / "blocks.bin").write_bytes(blocks.tobytes())
        run = subprocess.run([str(exe), str(fmt), str(tmp / "blocks.bin"), str(tmp / "rgba.bin"), str(w), str(h)],
                             capture_output=True, text=True, timeout=120)
        assert run.returncode == 0, run.stderr
        if fmt in (abi.BC6H_UF16, abi.BC6H_SF16):
            return np.fromfile(tmp / "rgba.bin", np.float32).reshape(h, w, 4)
        return np.fromfile(tmp / "rgba.bin", np.uint32).reshape(h, w)

    return decode


def test_bc7_oracle_matches_texture_unit(texture_unit):
    """Pins the BC7 oracle (and its partition, anchor and weight tables) to
    the GPU's texture unit: a BC7 CUDA array read through a point-sampled
    texture object decodes the same random blocks of every mode."""
    w, h = 256, 128  # 2,048 blocks, 256 per mode
    blocks = _bc7_blocks(np.random.default_rng(2024), (w // 4) * (h // 4), reserved=False)
    hw = texture_unit(abi.BC7, blocks, w, h)
    exp = ob.decode_bc(abi.BC7, blocks, w, h)
    bad = np.argwhere(hw != exp)
    if len(bad):
        by, bx = bad[0] // 4
        blk = blocks.reshape(h // 4, w // 4, 16)[by, bx]
        raise AssertionError(f"{len(bad)} texels differ; first at {tuple(bad[0])}: texture unit "
                             f"{hw[tuple(bad[0])]:08x}, oracle {exp[tuple(bad[0])]:08x}, block {blk.tobytes().hex()}")


# The 5-bit mode fields BC6H defines (0 and 1 are 2-bit modes), then the
# four reserved ones, which decode to 0.
_BC6H_MODES = [0x00, 0x01, 0x02, 0x06, 0x0A, 0x0E, 0x12, 0x16, 0x1A, 0x1E, 0x03, 0x07, 0x0B, 0x0F,
               0x13, 0x17, 0x1B, 0x1F]


def _bc6h_blocks(rng, n: int) -> np.ndarray:
    """n random BC6H blocks, every mode field value equally often: any bits
    after the mode field are a valid block."""
    blocks = rng.integers(0, 256, size=(n, 16), dtype=np.uint8)
    modes = np.array(_BC6H_MODES, np.uint8)[np.arange(n) % len(_BC6H_MODES)]
    rng.shuffle(modes)
    keep = np.where(modes < 2, 0xFC, 0xE0).astype(np.uint8)  # 2- or 5-bit field
    blocks[:, 0] = (blocks[:, 0] & keep) | modes
    return blocks.reshape(-1)


def _half_to_f32(bits: np.ndarray) -> np.ndarray:
    return bits.view(np.float16).astype(np.float32)


@pytest.mark.parametrize("fmt", [abi.BC6H_UF16, abi.BC6H_SF16])
@pytest.mark.parametrize("size", [(4, 4), (37, 21), (256, 128), (3, 5), (1024, 1000)])
def test_bc6h_decode_matches_oracle(renderer, fmt, size):
    """k_decode_bc6h's float32 RGB is the oracle's binary16 texels, bit for
    bit (signed zeros included), at block-aligned and ragged sizes."""
    w, h = size
    rng = np.random.default_rng(w * 13 + h + fmt)
    blocks = _bc6h_blocks(rng, ((w + 3) // 4) * ((h + 3) // 4))
    got = texture.decode_bc6h(renderer, fmt, blocks, w, h)
    torch.cuda.synchronize()
    exp = _half_to_f32(ob.decode_bc6h(blocks, w, h, fmt == abi.BC6H_SF16))
    assert np.array_equal(got.cpu().numpy().view(np.uint32), exp.view(np.uint32))


@pytest.mark.parametrize("fmt", [abi.BC6H_UF16, abi.BC6H_SF16])
def test_bc6h_oracle_matches_texture_unit(texture_unit, fmt):
    """Pins the BC6H oracle (its fourteen header layouts, sign extension,
    delta transform, unquantisation, weights and binary16 scaling) to the GPU
    texture unit's BC6H decode of the same random blocks of every mode."""
    w, h = 256, 144  # 2,304 blocks, 128 per mode field value
    blocks = _bc6h_blocks(np.random.default_rng(606 + fmt), (w // 4) * (h // 4))
    hw = texture_unit(fmt, blocks, w, h)
    assert (hw[..., 3] == 1.0).all()
    exp = ob.decode_bc6h(blocks, w, h, fmt == abi.BC6H_SF16)
    got = hw[..., :3].astype(np.float16).view(np.uint16)
    bad = np.argwhere((got != exp).any(axis=2))
    assert not len(bad), f"{len(bad)} texels differ; first at {tuple(bad[0])}"


def test_bc6h_through_load_image(renderer):
    """BC6H in a DDS (DX10 header, DXGI 95 / 96) and in a KTX2 (vkFormat 143
    / 144) decodes through load_image to the oracle's texels, float32 RGB."""
    from test_texture_decode import _dds, _ktx2

    blocks = _bc6h_blocks(np.random.default_rng(78), 10 * 6)
    for data, kind, signed in ((_dds(b"DX10", 37, 22, blocks.tobytes(), dxgi=95), abi.IMAGE_DDS, False),
                               (_dds(b"DX10", 37, 22, blocks.tobytes(), dxgi=96), abi.IMAGE_DDS, True),
                               (_ktx2(143, 37, 22, blocks.tobytes()), abi.IMAGE_KTX2, False),
                               (_ktx2(144, 37, 22, blocks.tobytes()), abi.IMAGE_KTX2, True)):
        got = texture.load_image(data, kind, renderer)
        assert got.dtype == np.float32 and got.shape == (22, 37, 3)
        exp = _half_to_f32(ob.decode_bc6h(blocks, 37, 22, signed))
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


# Largest per-channel difference between the texture unit and the pinned
# BC1-BC5 rounding, measured on GB300 (R, G, B, A): the formats leave the
# interpolation's precision to the implementation and the texture unit's is
# lower, while a layout error
# (index or endpoint order, mode switch, alpha source) moves channels by far
# more.
_BC_HW_BOUND = {abi.BC1: (1, 5, 1, 0), abi.BC2: (1, 5, 1, 0), abi.BC3: (1, 5, 1, 6), abi.BC4: (7, 0, 0, 0),
                abi.BC5: (7, 7, 0, 0)}


@pytest.mark.parametrize("fmt", sorted(_BC_HW_BOUND))
def test_bc1_to_bc5_layout_matches_texture_unit(texture_unit, fmt):
    """BC1-BC5 against the texture unit's own decode of the same random
    blocks (both endpoint orders): every channel within the measured
    rounding bound, the channels a format lacks exactly as the oracle
    writes them, and BC1's transparent texels (three-colour mode, code 3)
    identical."""
    w, h = 256, 128
    rng = np.random.default_rng(fmt)  # the sample the bounds were measured on
    bsize = 8 if fmt in (abi.BC1, abi.BC4) else 16
    blocks = rng.integers(0, 256, size=(w // 4) * (h // 4) * bsize, dtype=np.uint8)
    if fmt in (abi.BC1, abi.BC4):
        blocks[::16] = np.minimum(blocks[::16], 127)
    hw = texture_unit(fmt, blocks, w, h).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    exp = ob.decode_bc(fmt, blocks, w, h).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    worst = np.abs(hw - exp).reshape(-1, 4).max(axis=0)
    assert all(int(worst[c]) <= _BC_HW_BOUND[fmt][c] for c in range(4)), (worst, _BC_HW_BOUND[fmt])
    if fmt == abi.BC1:
        transparent = exp[..., 3] == 0
        assert transparent.any() and (hw[transparent] == 0).all()


@pytest.mark.parametrize("case", range(13))
@pytest.mark.parametrize("size", [(37, 45), (1, 1), (17, 64), (300, 517)])
def test_jpeg_pixels_match_oracle(renderer, case, size):
    """k_jpeg_idct + k_jpeg_color against the oracle, from the same
    coefficient planes: every sampling layout, grey, RGB, ragged sizes."""
    from jpeg_util import encode as jpeg_encode
    from test_jpeg import CASES, _image

    img = _image(*size, seed=case)
    data, _ = jpeg_encode(img, rng=np.random.default_rng(case), **CASES[case])
    j = texture.Jpeg(data)
    got = j.to_rgba(renderer)
    torch.cuda.synchronize()
    exp = ob.jpeg_rgba(j.info, [p.reshape(-1) for p in j.planes])
    assert np.array_equal(got.cpu().numpy().view(np.uint32)[..., 0], exp)


def test_ktx2_through_load_image(renderer):
    from test_texture_decode import _ktx2

    rng = np.random.default_rng(4)
    for vk, fmt, bsize in ((131, abi.BC1_OPAQUE, 8), (137, abi.BC3, 16), (141, abi.BC5, 16)):
        blocks = rng.integers(0, 256, 10 * 6 * bsize, dtype=np.uint8)
        got = texture.load_image(_ktx2(vk, 37, 22, blocks.tobytes()), abi.IMAGE_KTX2, renderer)
        assert np.array_equal(got.view(np.uint32)[..., 0], ob.decode_bc(fmt, blocks, 37, 22))


def test_bc7_through_load_image(renderer):
    """BC7 in a DDS (DX10 header, DXGI 98 / 99) and in a KTX2 (vkFormat 145 /
    146) decodes through load_image to the oracle's texels."""
    from test_texture_decode import _dds, _ktx2

    rng = np.random.default_rng(77)
    blocks = _bc7_blocks(rng, 10 * 6)
    exp = ob.decode_bc(abi.BC7, blocks, 37, 22)
    for data, kind in ((_dds(b"DX10", 37, 22, blocks.tobytes(), dxgi=98), abi.IMAGE_DDS),
                       (_dds(b"DX10", 37, 22, blocks.tobytes(), dxgi=99), abi.IMAGE_DDS),
                       (_ktx2(145, 37, 22, blocks.tobytes()), abi.IMAGE_KTX2),
                       (_ktx2(146, 37, 22, blocks.tobytes()), abi.IMAGE_KTX2)):
        got = texture.load_image(data, kind, renderer)
        assert np.array_equal(got.view(np.uint32)[..., 0], exp)


def test_zstd_ktx2_through_load_image(renderer):
    """Zstandard-supercompressed KTX2 levels (committed libzstd frames of
    block data) inflate on the host and decode on the device to the oracle's
    texels of the same blocks."""
    import base64
    import json
    import struct
    from pathlib import Path

    from test_texture_decode import _ktx2

    cases = json.loads((Path(__file__).resolve().parent / "golden" / "zstd_frames.json").read_text())["cases"]
    used = 0
    for c in cases:
        if c["name"] != "bc1_blocks":
            continue
        frame = base64.b64decode(c["frame"])
        blocks = np.frombuffer(texture.zstd_decompress(frame, c["size"]).tobytes(), np.uint8)
        bw = 32
        bh = c["size"] // (8 * bw)
        data = bytearray(_ktx2(133, 4 * bw, 4 * bh, frame, scheme=2))
        struct.pack_into("<Q", data, 96, bw * bh * 8)  # uncompressedByteLength
        got = texture.load_image(bytes(data), abi.IMAGE_KTX2, renderer)
        assert np.array_equal(got.view(np.uint32)[..., 0], ob.decode_bc(abi.BC1, blocks[: bw * bh * 8], 4 * bw, 4 * bh))
        used += 1
    assert used == 3


def test_jpeg_through_load_image_and_freed_source(renderer):
    """decode_jpeg frees the host coefficients before the device finishes:
    the copy is staged, so the pixels are still the oracle's."""
    from jpeg_util import encode as jpeg_encode
    from test_jpeg import _image

    img = _image(1024, 768, seed=3)
    data, _ = jpeg_encode(img, rng=np.random.default_rng(1), sampling=((2, 2), (1, 1), (1, 1)), restart=7)
    outs = [texture.decode_jpeg(data, renderer) for _ in range(3)]  # scratch reuse across calls
    torch.cuda.synchronize()
    j = texture.Jpeg(data)
    exp = ob.jpeg_rgba(j.info, [p.reshape(-1) for p in j.planes])
    for o in outs:
        assert np.array_equal(o.cpu().numpy().view(np.uint32)[..., 0], exp)
    via = texture.load_image(data, abi.IMAGE_JPEG, renderer)
    assert np.array_equal(via.view(np.uint32)[..., 0], exp)
    # the same image as a progressive file: the same coefficients, so the same pixels
    prog, _ = jpeg_encode(img, rng=np.random.default_rng(1), sampling=((2, 2), (1, 1), (1, 1)), restart=7,
                          progressive=True)
    got = texture.decode_jpeg(prog, renderer)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy().view(np.uint32)[..., 0], exp)


@pytest.mark.parametrize("dds_format", ["bc3", "bc6h"])
def test_gltf_with_dds_and_png_textures(renderer, tmp_path, dds_format):
    """The DDS texture is BC3 (an RGBA8 texture) or BC6H UF16 (a linear
    float32 RGB texture)."""
    base = small_grid()
    mesh = base.meshes[0]
    world = grid_world(mesh.meshlet_count, mesh.position_scale, grid=(4, 4, 2), animated=False)
    rng = np.random.default_rng(5)
    b = Builder()
    pos = b.accessor(mesh.positions.astype(np.float32))
    uv = b.accessor(mesh.uvs.astype(np.float32))
    idx = b.accessor(mesh.indices.reshape(-1).astype(np.uint32))
    for material in (0, 1):  # mesh 0 uses the DDS texture, mesh 1 the PNG one
        b.add("meshes", {"primitives": [{"attributes": {"POSITION": pos, "TEXCOORD_0": uv}, "indices": idx,
                                         "material": material}]})
    if dds_format == "bc3":
        dds_blocks = rng.integers(0, 256, size=16 * 16 * 16, dtype=np.uint8)  # 64 x 64 texels of BC3
        dds = _dds(b"DXT5", 64, 64, dds_blocks.tobytes())
    else:
        dds_blocks = _bc6h_blocks(rng, 16 * 16)  # 64 x 64 texels of BC6H UF16
        dds = _dds(b"DX10", 64, 64, dds_blocks.tobytes(), dxgi=95)
    png_pixels = rng.integers(0, 256, size=(32, 48, 4))
    png = encode(png_pixels, 6, 8, rng)
    img_dds = b.add("images", {"bufferView": b._view(dds), "mimeType": "image/vnd-ms.dds"})
    img_png = b.add("images", {"bufferView": b._view(png), "mimeType": "image/png"})
    b.add("textures", {"source": img_png, "extensions": {"MSFT_texture_dds": {"source": img_dds}}})
    b.add("textures", {"source": img_png})
    xf = {"KHR_texture_transform": {"scale": [4.0, 4.0]}}
    b.add("materials", {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0, "extensions": xf}}})
    b.add("materials", {"pbrMetallicRoughness": {"baseColorTexture": {"index": 1, "extensions": xf}}})
    for k, n in enumerate(world.nodes):
        node = {"translation": [float(x) for x in n["translation"]], "rotation": [float(x) for x in n["rotation"]],
                "scale": [float(x) for x in n["scale"]]}
        if n["mesh_index"] != abi.INVALID_HANDLE:
            node["mesh"] = k % 2
        f, c = int(n["first_child"]), int(n["child_count"])
        if c:
            node["children"] = [int(x) for x in world.children[f:f + c]]
        b.add("nodes", node)
    b.gltf["scenes"] = [{"nodes": [int(r) for r in world.roots]}]
    path = b.write_glb(tmp_path / "textured.glb")

    host, iworld = gltf.load(path, images=True, renderer=renderer)
    assert len(host.textures) == 2
    if dds_format == "bc3":
        assert host.textures[0].format == abi.TEXTURE_RGBA8
        assert np.array_equal(host.textures[0].data.reshape(64, 64, 4).view(np.uint32)[..., 0],
                              ob.decode_bc(abi.BC3, dds_blocks, 64, 64))
    else:
        assert host.textures[0].format == abi.TEXTURE_RGB32F
        exp = _half_to_f32(ob.decode_bc6h(dds_blocks, 64, 64, False))
        assert np.array_equal(host.textures[0].data.view(np.uint32), exp.view(np.uint32))
    assert np.array_equal(host.textures[1].data, png_pixels.astype(np.uint8))
    assert host.materials[1]["albedo_index"] == 0 and host.materials[2]["albedo_index"] == 1
    dev, dw = gltf.device_scene(renderer, host, iworld)
    try:
        ohost = dataclasses.replace(host, transforms=ob.world_transforms(iworld, 0.0), draws=ob.world_draws(iworld))
        osc = ob.OracleScene(ohost)
        centre = scene.grid_centre() * 0.25
        eye = centre + np.array([6.0, 5.0, 7.0])
        cam = scene.camera(tuple(eye), tuple(centre), scene.safe_up(eye, centre), 70.0, 1.6)
        flags = abi.CULL_FRUSTUM | abi.RESOLVE_TEXTURED | abi.WRITE_IDS
        v = ViewBuffers.allocate(320, 200, cam, host.draw_count)
        renderer.frame(dev, [v], flags)
        torch.cuda.synchronize()
        e = ob.frame(osc, cam, 320, 200, oracle_flags(flags))
        assert (u64(v.depth_id) != 0).sum() > 2000
        assert np.array_equal(u32(v.visbuffer), e["ids"])
        ok, bad = rgba_close(u32(v.color), e["rgba"])
        assert ok, bad
        # both primitives (DDS and PNG materials) are on screen
        prims = {int(host.draws[i >> 7][0]) for i in np.unique(u32(v.visbuffer)) if i != 0xFFFFFFFF}
        assert prims == {0, 1}
    finally:
        dw.close()
