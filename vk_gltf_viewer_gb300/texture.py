"""Base-colour images for the textured resolve (``vkgv_image_*``,
``vkgv_dds_parse``, ``vkgv_decode_bc``, ``vkgv_decode_bc6h``).

PNG decodes on the host into RGBA8; DDS and KTX2 files hold BC1-BC5 or BC7
blocks, which the device decodes into RGBA8, or BC6H blocks, which it
decodes into float32 RGB (a linear ``TEXTURE_RGB32F`` texture); JPEG is
entropy-decoded on the host and turned into pixels on the device.  The
reference loads no images (src/vk_gltf_viewer/assets.cpp:467-471).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi
from .renderer import _stream_handle


def decode_png(data: bytes) -> np.ndarray:
    """PNG bytes -> (H, W, 4) uint8 RGBA."""
    lib = abi.load()
    buf = np.frombuffer(data, np.uint8)
    h = C.c_void_p()
    err = C.create_string_buffer(256)
    rc = lib.vkgv_image_decode_png(buf.ctypes.data, buf.size, C.byref(h), err, len(err))
    if rc != abi.OK:
        raise abi.VkgvError(rc, err.value.decode(errors="replace"))
    try:
        w, hh, px = C.c_uint32(), C.c_uint32(), C.c_void_p()
        abi.check(lib.vkgv_image_get(h, C.byref(w), C.byref(hh), C.byref(px)))
        n = w.value * hh.value * 4
        return np.frombuffer(C.string_at(px.value, n), np.uint8).reshape(hh.value, w.value, 4).copy()
    finally:
        lib.vkgv_image_free(h)


def parse_dds(data: bytes) -> tuple[abi.DdsInfo, np.ndarray]:
    """DDS bytes -> (header info, the top mip's block bytes)."""
    buf = np.frombuffer(data, np.uint8)
    info = abi.DdsInfo()
    rc = abi.load().vkgv_dds_parse(buf.ctypes.data, buf.size, C.byref(info))
    if rc != abi.OK:
        raise abi.VkgvError(rc, "not a DDS file with BC1-BC5, BC6H, BC7 or 32-bit RGBA / BGRA data")
    blocks = buf[info.data_offset:info.data_offset + info.data_size].copy()
    return info, blocks


def zstd_decompress(data, size: int) -> np.ndarray:
    """Zstandard frames -> exactly `size` decoded bytes (vkgv_zstd_decompress)."""
    src = np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else np.ascontiguousarray(data, np.uint8)
    out = np.empty(max(1, size), np.uint8)
    n = C.c_uint64()
    rc = abi.load().vkgv_zstd_decompress(src.ctypes.data, src.size, out.ctypes.data, size, C.byref(n))
    if rc != abi.OK:
        raise abi.VkgvError(rc, "corrupt Zstandard data, or more than the expected size")
    if n.value != size:
        raise abi.VkgvError(abi.INVALID_ARG, f"Zstandard data decoded to {n.value} bytes, expected {size}")
    return out[:size]


def parse_ktx2(data: bytes) -> tuple[abi.DdsInfo, np.ndarray]:
    """KTX2 bytes -> (header info, level 0's bytes): BC1-BC5 blocks or
    RGBA8 texels (``info.format`` is ``abi.RGBA8`` for those), inflated
    first when the level is Zstandard-supercompressed."""
    buf = np.frombuffer(data, np.uint8)
    info = abi.DdsInfo()
    rc = abi.load().vkgv_ktx2_parse(buf.ctypes.data, buf.size, C.byref(info))
    if rc != abi.OK:
        raise abi.VkgvError(rc, "not a KTX2 file with BC1-BC5, BC6H, BC7 or RGBA8 data, uncompressed or Zstandard-"
                                "supercompressed (BasisU files are not decoded)")
    level = buf[info.data_offset:info.data_offset + info.data_size]
    if info.supercompression == 2:
        if info.format == abi.RGBA8:
            size = info.width * info.height * 4
        else:
            block = 8 if info.format in (abi.BC1, abi.BC4, abi.BC1_OPAQUE) else 16
            size = ((info.width + 3) // 4) * ((info.height + 3) // 4) * block
        return info, zstd_decompress(level, size)
    return info, level.copy()


def decode_bc(renderer, fmt: int, blocks, width: int, height: int, stream=None) -> torch.Tensor:
    """BC1-BC5 blocks -> device (height, width, 4) uint8 RGBA, decoded by
    k_decode_bc.  `blocks` is a numpy array or a device tensor of bytes."""
    dev = torch.device("cuda", renderer.device)
    if isinstance(blocks, np.ndarray):
        blocks = torch.from_numpy(np.ascontiguousarray(blocks, np.uint8)).to(dev)
    out = torch.empty((height, width, 4), dtype=torch.uint8, device=blocks.device)
    abi.check(abi.load().vkgv_decode_bc(renderer.ctx, fmt, blocks.data_ptr(), width, height, out.data_ptr(),
                                        _stream_handle(stream)), renderer.ctx)
    return out


def decode_bc6h(renderer, fmt: int, blocks, width: int, height: int, stream=None) -> torch.Tensor:
    """BC6H blocks (``abi.BC6H_UF16`` or ``abi.BC6H_SF16``) -> device
    (height, width, 3) float32 RGB, the format's binary16 values exactly,
    decoded by k_decode_bc6h.  `blocks` is a numpy array or a device tensor
    of bytes."""
    dev = torch.device("cuda", renderer.device)
    if isinstance(blocks, np.ndarray):
        blocks = torch.from_numpy(np.ascontiguousarray(blocks, np.uint8)).to(dev)
    out = torch.empty((height, width, 3), dtype=torch.float32, device=blocks.device)
    abi.check(abi.load().vkgv_decode_bc6h(renderer.ctx, fmt, blocks.data_ptr(), width, height, out.data_ptr(),
                                          _stream_handle(stream)), renderer.ctx)
    return out


def _uncompressed_dds(info, texels: np.ndarray) -> np.ndarray:
    """32-bit DDS texels -> (H, W, 4) uint8 RGBA: B, G, R byte orders
    swapped, a fourth byte that is not alpha read as 255."""
    px = np.array(texels, np.uint8).reshape(info.height, info.width, 4)
    if info.format in (abi.BGRA8, abi.BGRX8):
        px = px[..., [2, 1, 0, 3]].copy()
    if info.format in (abi.RGBX8, abi.BGRX8):
        px[..., 3] = 255
    return px


def _decode_blocks(renderer, info, blocks) -> np.ndarray:
    if info.format in (abi.BC6H_UF16, abi.BC6H_SF16):
        img = decode_bc6h(renderer, info.format, blocks, info.width, info.height)
    else:
        img = decode_bc(renderer, info.format, blocks, info.width, info.height)
    torch.cuda.synchronize()
    return img.cpu().numpy()


class Jpeg:
    """A JPEG's entropy decode (host): ``info`` (``abi.JpegInfo``) and its
    dequantized coefficient planes, ``planes[c]`` of shape
    (blocks_h, blocks_w, 8, 8) int16 in natural order.  ``to_rgba`` runs the
    IDCT, upsampling and colour conversion on the device."""

    def __init__(self, data: bytes):
        self._h = None
        lib = abi.load()
        buf = np.frombuffer(data, np.uint8)
        h = C.c_void_p()
        err = C.create_string_buffer(256)
        rc = lib.vkgv_jpeg_decode_coefficients(buf.ctypes.data, buf.size, C.byref(h), err, len(err))
        if rc != abi.OK:
            raise abi.VkgvError(rc, err.value.decode(errors="replace"))
        self._h = h
        self.info = abi.JpegInfo()
        abi.check(lib.vkgv_jpeg_get_info(h, C.byref(self.info)))

    @property
    def planes(self) -> list[np.ndarray]:
        lib, out = abi.load(), []
        for c in range(self.info.components):
            ptr = C.c_void_p()
            abi.check(lib.vkgv_jpeg_get_coefficients(self._h, c, C.byref(ptr)))
            bw, bh = self.info.blocks_w[c], self.info.blocks_h[c]
            out.append(np.frombuffer(C.string_at(ptr.value, bw * bh * 128), np.int16).reshape(bh, bw, 8, 8).copy())
        return out

    def to_rgba(self, renderer, stream=None) -> torch.Tensor:
        """Device (height, width, 4) uint8 RGBA."""
        out = torch.empty((self.info.height, self.info.width, 4), dtype=torch.uint8,
                          device=torch.device("cuda", renderer.device))
        abi.check(abi.load().vkgv_jpeg_to_rgba(renderer.ctx, self._h, out.data_ptr(), _stream_handle(stream)),
                  renderer.ctx)
        return out

    def close(self):
        if self._h:
            abi.load().vkgv_jpeg_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def decode_jpeg(data: bytes, renderer, stream=None) -> torch.Tensor:
    """JPEG bytes -> device (H, W, 4) uint8 RGBA (entropy decode on the host,
    the pixels on the device)."""
    j = Jpeg(data)
    try:
        return j.to_rgba(renderer, stream)
    finally:
        j.close()


def load_image(data: bytes, kind: int, renderer=None) -> np.ndarray:
    """Encoded image -> host (H, W, 4) uint8 RGBA, or (H, W, 3) float32 RGB
    for BC6H: PNG, RGBA8 KTX2 and uncompressed DDS on the host;
    block-compressed DDS and KTX2, and JPEG, on the device (they need a
    renderer)."""
    if kind == abi.IMAGE_PNG:
        return decode_png(data)
    if kind == abi.IMAGE_DDS:
        info, blocks = parse_dds(data)
        if info.format in (abi.RGBA8, abi.BGRA8, abi.RGBX8, abi.BGRX8):
            return _uncompressed_dds(info, blocks)
        if renderer is None:
            raise ValueError("block-compressed DDS images decode on the device: pass a renderer")
        return _decode_blocks(renderer, info, blocks)
    if kind == abi.IMAGE_JPEG:
        if renderer is None:
            raise ValueError("JPEG images decode on the device: pass a renderer")
        img = decode_jpeg(data, renderer)
        torch.cuda.synchronize()
        return img.cpu().numpy()
    if kind == abi.IMAGE_KTX2:
        info, payload = parse_ktx2(data)
        if info.format == abi.RGBA8:
            return payload.reshape(info.height, info.width, 4)
        if renderer is None:
            raise ValueError("KTX2 block-compressed images decode on the device: pass a renderer")
        return _decode_blocks(renderer, info, payload)
    raise abi.VkgvError(abi.INVALID_ARG, "unknown image format")
