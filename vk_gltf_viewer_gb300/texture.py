"""Base-colour images for the textured resolve (``vkgv_image_*``,
``vkgv_dds_parse``, ``vkgv_decode_bc``).

PNG decodes on the host into RGBA8; DDS files hold BC1-BC5 blocks, which the
device decodes into RGBA8.  The reference loads no images
(src/vk_gltf_viewer/assets.cpp:467-471).
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
        raise abi.VkgvError(rc, "not a DDS file with BC1-BC5 data")
    blocks = buf[info.data_offset:info.data_offset + info.data_size].copy()
    return info, blocks


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


def load_image(data: bytes, kind: int, renderer=None) -> np.ndarray:
    """Encoded image -> host (H, W, 4) uint8 RGBA: PNG on the host, DDS on
    the device (needs a renderer)."""
    if kind == abi.IMAGE_PNG:
        return decode_png(data)
    if kind == abi.IMAGE_DDS:
        if renderer is None:
            raise ValueError("DDS images decode on the device: pass a renderer")
        info, blocks = parse_dds(data)
        img = decode_bc(renderer, info.format, blocks, info.width, info.height)
        torch.cuda.synchronize()
        return img.cpu().numpy()
    names = {abi.IMAGE_JPEG: "JPEG", abi.IMAGE_KTX2: "KTX2"}
    raise abi.VkgvError(abi.INVALID_ARG, f"{names.get(kind, 'unknown')} images are not decoded")
