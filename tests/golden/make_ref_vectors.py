"""Writes tests/golden/ref_headers.json from the reference's own shared GLSL
headers compiled in their C++ mode (oracle/ref_shim.cpp, built from the
reference sources by `make -C oracle ref`): the struct sizes, member offsets
and constants of shaders/mesh_common.h.glsl:20-126 and
shaders/visbuffer/visbuffer.h.glsl:15-67, and fromLinear / toLinear of
shaders/srgb.h.glsl:9-41 (scalar and vec4 forms) on a fixed sweep of inputs
(binary32 bits).

Run where the reference sources are present:
    python tests/golden/make_ref_vectors.py
The fixture lets the tests check the oracle and the library against the
reference's own code on machines without the reference sources."""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import binding  # noqa: E402


def srgb_sweep() -> np.ndarray:
    """Inputs: a uniform sweep of [0, 1], dense samples around both cut-offs
    (0.0031308 and 0.04045), the binary32 neighbours of the cut-offs, and
    the ends."""
    xs = [np.linspace(0.0, 1.0, 769, dtype=np.float32),
          np.linspace(0.0025, 0.0037, 96, dtype=np.float32),
          np.linspace(0.039, 0.042, 96, dtype=np.float32)]
    edge = []
    for c in (np.float32(0.0031308), np.float32(0.04045)):
        b = int(c.view(np.uint32))
        edge += [np.uint32(b + k).view(np.float32) for k in range(-4, 5)]
    xs.append(np.array(edge + [0.0, 1e-6, 0.5, 1.0], np.float32))
    return np.unique(np.concatenate(xs)).astype(np.float32)


def main():
    lib = binding.load_ref()
    if lib is None:
        raise SystemExit("the reference sources are needed to build oracle/_ref")
    import ctypes as C
    xs = srgb_sweep()
    fl = np.array([lib.ref_from_linear(float(x)) for x in xs], np.float32)
    tl = np.array([lib.ref_to_linear(float(x)) for x in xs], np.float32)
    # the vec4 forms (srgb.h.glsl:26-41), which the resolve calls on the
    # albedo (visbuffer_resolve.comp.glsl:38): each input in r, g and b
    # (alpha passes through unchanged)
    fl4 = np.zeros(xs.size, np.float32)
    tl4 = np.zeros(xs.size, np.float32)
    out = np.zeros(4, np.float32)
    for i, x in enumerate(xs):
        v = np.array([x, x, x, 0.25], np.float32)
        lib.ref_from_linear4(v.ctypes.data, out.ctypes.data)
        assert out[0] == out[1] == out[2] and out[3] == np.float32(0.25)
        fl4[i] = out[0]
        lib.ref_to_linear4(v.ctypes.data, out.ctypes.data)
        assert out[0] == out[1] == out[2] and out[3] == np.float32(0.25)
        tl4[i] = out[0]
    packs = []
    rng = np.random.default_rng(5)
    for d, t in [(0, 0), (1, 0), (0, 127), (12345, 77), ((1 << 25) - 1, 127)] + \
            [(int(a), int(b)) for a, b in zip(rng.integers(0, 1 << 25, 27), rng.integers(0, 128, 27))]:
        v = int(lib.ref_pack_visbuffer(d, t))
        dd, tt = C.c_uint32(), C.c_uint32()
        lib.ref_unpack_visbuffer(v, C.byref(dd), C.byref(tt))
        packs.append([d, t, v, int(dd.value), int(tt.value)])
    result = {
        "source": "reference shaders/mesh_common.h.glsl, shaders/visbuffer/visbuffer.h.glsl, shaders/srgb.h.glsl "
                  "compiled in their C++ mode (oracle/ref_shim.cpp)",
        "layout": binding.ref_layout(lib),
        "srgb_inputs": [int(x) for x in xs.view(np.uint32)],
        "from_linear": [int(x) for x in fl.view(np.uint32)],
        "to_linear": [int(x) for x in tl.view(np.uint32)],
        "from_linear4": [int(x) for x in fl4.view(np.uint32)],
        "to_linear4": [int(x) for x in tl4.view(np.uint32)],
        "pack": packs,
    }
    path = Path(__file__).resolve().parent / "ref_headers.json"
    path.write_text(json.dumps(result, separators=(",", ":")) + "\n")
    print(f"wrote {path} ({path.stat().st_size} bytes, {xs.size} sRGB inputs)")


if __name__ == "__main__":
    main()
