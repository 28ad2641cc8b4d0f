"""JPEG decoding (the reference links wuffs for JPEG, its image task is
empty: src/vk_gltf_viewer/assets.cpp:467-471).  The host entropy decoder
returns exactly the dequantized coefficients a T.81 encoder wrote, for grey,
YCbCr and RGB files, every sampling layout, 8- and 16-bit tables, restart
intervals and single-component scans, sequential or progressive; the
oracle's fixed-point IDCT is pinned against the float64 inverse DCT;
malformed files fail with a message."""
import math

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, texture

from jpeg_util import encode

CASES = [
    dict(mode="ycc"),
    dict(mode="ycc", sampling=((2, 2), (1, 1), (1, 1))),
    dict(mode="ycc", sampling=((2, 1), (1, 1), (1, 1)), restart=2),
    dict(mode="ycc", sampling=((1, 2), (1, 1), (1, 1)), restart=1),
    dict(mode="ycc", sampling=((2, 2), (1, 1), (1, 1)), interleaved=False, restart=5),
    dict(mode="ycc", sampling=((4, 1), (2, 1), (1, 1))),
    dict(mode="ycc", sampling=((1, 1), (2, 2), (1, 1))),  # a chroma plane sampled above luma
    dict(mode="gray"),
    dict(mode="gray", restart=3),
    dict(mode="rgb"),
    dict(mode="rgb", rgb_ids=True, qt16=True),
    dict(mode="ycc", quality=40),
    dict(mode="ycc", quality=100),
]


def _image(h, w, seed, noise=0.2):
    """Gradients with a fraction of random pixels (long Huffman codes)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    smooth = np.stack([(x * 5 + y) % 256, (y * 7) % 256, ((x + y) * 3) % 256], -1)
    return np.where(rng.random((h, w, 1)) < noise, rng.integers(0, 256, (h, w, 3)), smooth).astype(np.uint8)


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("size", [(37, 45), (8, 8), (1, 1), (17, 64)])
def test_coefficients_round_trip(built, case, size):
    kw = CASES[case]
    img = _image(*size, seed=case)
    data, expected = encode(img, rng=np.random.default_rng(case), **kw)
    j = texture.Jpeg(data)
    assert (j.info.width, j.info.height) == (size[1], size[0])
    assert j.info.components == (1 if kw["mode"] == "gray" else 3)
    assert j.info.rgb == (kw["mode"] == "rgb")
    got = j.planes
    assert len(got) == len(expected)
    for g, e in zip(got, expected):
        assert np.array_equal(g, e)


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("size", [(37, 45), (1, 1), (70, 90)])
@pytest.mark.parametrize("seed", [0, 1])
def test_progressive_coefficients_round_trip(built, case, size, seed):
    """SOF2 files: DC first / refinement scans (interleaved or not), AC bands
    with successive approximation, end-of-band runs of random lengths and
    restart intervals decode to exactly the coefficients encoded."""
    kw = CASES[case]
    img = _image(*size, seed=case)
    data, expected = encode(img, rng=np.random.default_rng(seed * 100 + case), progressive=True, **kw)
    assert data[data.index(b"\xff\xc2"):][:2] == b"\xff\xc2"
    got = texture.Jpeg(data).planes
    for g, e in zip(got, expected):
        assert np.array_equal(g, e)


def test_oracle_idct_is_the_inverse_dct(built):
    """The pinned fixed-point IDCT is within 1 of the float64 inverse DCT
    rounded, on random and extreme blocks (constants derived in the oracle)."""
    rng = np.random.default_rng(3)
    blocks = rng.integers(-300, 300, (64, 8, 8)).astype(np.int16)
    blocks[:8, 0, 0] = [-1024, 1016, 0, 512, -512, 8, -8, 1]
    blocks[8] = 0
    blocks[9, 7, 7] = 1000
    c = np.array([[(1 / math.sqrt(2) if u == 0 else 1.0) / 2 * math.cos((2 * x + 1) * u * math.pi / 16)
                   for u in range(8)] for x in range(8)])
    ref = np.einsum("xu,yv,bvu->byx", c, c, blocks.astype(np.float64)) + 128
    ref = np.clip(np.round(ref), 0, 255)

    class Info:
        width, height, components, rgb, hmax, vmax = 8 * 64, 8, 1, 0, 1, 1
        h = v = (1, 1, 1)
        blocks_w, blocks_h = (64, 1, 1), (1, 1, 1)
    out = ob.jpeg_rgba(Info, [blocks.reshape(-1)]).view(np.uint8).reshape(8, 64 * 8, 4)[..., 0]
    got = out.reshape(8, 64, 8).transpose(1, 0, 2)
    assert np.abs(got.astype(int) - ref).max() <= 1


def test_oracle_pixels_approximate_the_source(built):
    y, x = np.mgrid[0:48, 0:64]
    img = np.stack([x * 3, y * 4, (x + y) * 2], -1).astype(np.uint8)  # smooth: subsampling keeps it
    for kw, tol in ((dict(mode="ycc", quality=95), 1.5), (dict(mode="gray", quality=95), 1.0),
                    (dict(mode="ycc", sampling=((2, 2), (1, 1), (1, 1)), quality=95), 2.5)):
        data, _ = encode(img, rng=np.random.default_rng(2), **kw)
        j = texture.Jpeg(data)
        px = ob.jpeg_rgba(j.info, [p.reshape(-1) for p in j.planes]).view(np.uint8).reshape(48, 64, 4)
        ref = img if kw["mode"] != "gray" else np.repeat(img[..., :1], 3, -1)
        assert np.abs(px[..., :3].astype(int) - ref).mean() < tol
        assert (px[..., 3] == 255).all()


def _first(data: bytes, marker: int) -> int:
    return data.index(bytes([0xFF, marker]))


def test_errors(built):
    img = _image(20, 24, 1)
    data, _ = encode(img, rng=np.random.default_rng(0), restart=2)
    sos = _first(data, 0xDA)
    cases = {
        "not a JPEG": b"\x89PNG" + data[4:],
        "DC coefficient only": data.replace(b"\xff\xc0", b"\xff\xc2", 1),  # a sequential scan in SOF2
        "differential": data.replace(b"\xff\xc0", b"\xff\xc6", 1),
        "arithmetic": data.replace(b"\xff\xc0", b"\xff\xc9", 1),
        "ends early": data[:sos + 40],
        "restart marker": data.replace(b"\xff\xd1", b"\xff\xd3", 1),
        "scan before the frame": data[:2] + data[sos:],
    }
    sof = _first(data, 0xC0)
    twelve = bytearray(data)
    twelve[sof + 4] = 12
    cases["8-bit"] = bytes(twelve)
    huge = bytearray(data)  # a 16000 x 16000 frame over a few hundred bytes of data
    huge[sof + 5:sof + 9] = bytes([0x3E, 0x80, 0x3E, 0x80])
    cases["too short"] = bytes(huge)
    # a DHT with three 1-bit codes: refused before its third code is placed
    # (it would index past the 9-bit lookahead table)
    dht = bytes([0xFF, 0xC4, 0x00, 2 + 17 + 3, 0x00, 3] + [0] * 15 + [1, 2, 3])
    cases["over-subscribed"] = data[:2] + dht + data[2:]
    for match, bad in cases.items():
        with pytest.raises(abi.VkgvError, match=match):
            texture.Jpeg(bad)
    # T.81 allows at most 10 blocks in an interleaved MCU (4x2 + 2x1 + 1 = 11)
    wide, _ = encode(img, rng=np.random.default_rng(0), sampling=((4, 2), (2, 1), (1, 1)))
    with pytest.raises(abi.VkgvError, match="10 blocks"):
        texture.Jpeg(wide)
    # a missing EOI is accepted: the scans are complete
    assert texture.Jpeg(data[:-2]).info.width == 24


@pytest.mark.parametrize("progressive", [False, True])
def test_restart_intervals_decoded_on_threads(built, progressive):
    """Enough restart intervals for the threaded entropy decode (runs of
    intervals on several threads): the same coefficients, and a restart
    marker out of order or a damaged interval still fails."""
    img = _image(512, 384, seed=3)
    data, expected = encode(img, rng=np.random.default_rng(5), sampling=((2, 2), (1, 1), (1, 1)), restart=3,
                            progressive=progressive)
    for g, e in zip(texture.Jpeg(data).planes, expected):
        assert np.array_equal(g, e)
    # the 40th restart marker of the first scan renumbered
    sos = data.index(b"\xff\xda")
    at, k = sos, 0
    while k < 40:
        at = data.index(b"\xff", at + 1)
        if 0xD0 <= data[at + 1] <= 0xD7:
            k += 1
    bad = bytearray(data)
    bad[at + 1] = 0xD0 + ((bad[at + 1] - 0xD0 + 3) & 7)
    with pytest.raises(abi.VkgvError, match="restart marker"):
        texture.Jpeg(bytes(bad))
    # entropy bytes of a middle interval damaged: an error, never a crash
    bad = bytearray(data)
    for j in range(at - 12, at - 2):
        if bad[j] not in (0xFF, 0x00):
            bad[j] ^= 0x5A
    try:
        texture.Jpeg(bytes(bad)).close()
    except abi.VkgvError:
        pass
