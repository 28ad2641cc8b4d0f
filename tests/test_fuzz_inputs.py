"""Malformed inputs to the host-side readers (glTF JSON / GLB with and
without EXT_meshopt_compression, PNG / DEFLATE, JPEG, KTX2, DDS): seeded byte mutations, truncations and insertions of valid files
either load or fail with a status, in a child process so that a crash or a
hang would fail the test instead of the run."""
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = textwrap.dedent("""
    import sys
    from pathlib import Path
    sys.path.insert(0, {root!r})
    sys.path.insert(0, {tests!r})
    import numpy as np
    from vk_gltf_viewer_gb300 import abi, gltf, texture
    kind, path, seed, n = sys.argv[1], Path(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4])
    good = path.read_bytes()
    rng = np.random.default_rng(seed)
    ok = failed = 0
    for i in range(n):
        data = bytearray(good)
        op = rng.integers(0, 4)
        if op == 0:      # flip bytes
            for _ in range(int(rng.integers(1, 8))):
                data[int(rng.integers(0, len(data)))] ^= int(rng.integers(1, 256))
        elif op == 1:    # truncate
            data = data[: int(rng.integers(0, len(data)))]
        elif op == 2:    # insert junk
            at = int(rng.integers(0, len(data)))
            data[at:at] = bytes(rng.integers(0, 256, int(rng.integers(1, 64)), dtype=np.uint8))
        else:            # overwrite a run with a digit or bracket (JSON structure)
            at = int(rng.integers(0, len(data)))
            data[at:at + 4] = bytes([b"0123456789[]{{}}\\",:"[int(rng.integers(0, 16))]]) * 4
        try:
            if kind in ("glb", "gltf", "meshopt"):
                out = path.with_name("mut." + ("glb" if kind == "meshopt" else kind))
                out.write_bytes(bytes(data))
                gltf.load(out, images=False)
            elif kind == "png":
                texture.decode_png(bytes(data))
            elif kind in ("jpeg", "jpeg_progressive"):
                texture.Jpeg(bytes(data)).close()
            elif kind == "ktx2":
                texture.parse_ktx2(bytes(data))
            else:
                texture.parse_dds(bytes(data))
            ok += 1
        except (abi.VkgvError, ValueError):
            failed += 1
    print(ok, failed)
""")


def _asset(tmp_path):
    from vk_gltf_viewer_gb300.gltf_export import Builder
    from vk_gltf_viewer_gb300 import scene
    from vk_gltf_viewer_gb300.world import grid_world

    b = Builder()
    ico = scene.icosphere(1)
    b.add("meshes", {"primitives": [{"attributes": {"POSITION": b.accessor(ico.positions.astype(np.float32))},
                                     "indices": b.accessor(ico.indices.reshape(-1).astype(np.uint16))}]})
    b.add("nodes", {"mesh": 0, "children": [1], "rotation": [0, 0.6, 0, 0.8]})
    b.add("nodes", {"mesh": 0, "translation": [1, 2, 3]})
    b.gltf["scenes"] = [{"nodes": [0]}]
    t = b.accessor(np.array([0.0, 1.0], np.float32))
    b.add("animations", {"samplers": [{"input": t, "output": b.accessor(np.zeros((2, 3), np.float32))}],
                         "channels": [{"sampler": 0, "target": {"node": 1, "path": "translation"}}]})
    return b


@pytest.mark.parametrize("kind", ["glb", "gltf", "meshopt", "png", "jpeg", "jpeg_progressive", "ktx2", "dds"])
def test_mutated_inputs_fail_cleanly(built, tmp_path, kind):
    if kind == "meshopt":  # EXT_meshopt_compression streams in the GLB's binary chunk
        from test_meshopt import _scene_builder
        path = _scene_builder(True, np.random.default_rng(2)).write_glb(tmp_path / "m.glb")
    elif kind == "glb":
        path = _asset(tmp_path).write_glb(tmp_path / "a.glb")
    elif kind == "gltf":
        path = _asset(tmp_path).write_gltf(tmp_path / "a.gltf")
    elif kind in ("jpeg", "jpeg_progressive"):
        from jpeg_util import encode as jpeg_encode
        rng = np.random.default_rng(0)
        path = tmp_path / "a.jpg"
        path.write_bytes(jpeg_encode(rng.integers(0, 256, (19, 27, 3)), sampling=((2, 2), (1, 1), (1, 1)),
                                     restart=2, progressive=kind == "jpeg_progressive", rng=rng)[0])
    elif kind == "ktx2":
        from test_texture_decode import _ktx2
        path = tmp_path / "a.ktx2"
        path.write_bytes(_ktx2(137, 12, 8, bytes(range(96))))
    elif kind == "png":
        from png_util import encode
        rng = np.random.default_rng(0)
        path = tmp_path / "a.png"
        path.write_bytes(encode(rng.integers(0, 256, (17, 23, 4)), 6, 8, rng, interlace=True))
    else:
        from test_texture_decode import _dds
        path = tmp_path / "a.dds"
        path.write_bytes(_dds(b"DXT5", 12, 8, bytes(range(96))))
    script = tmp_path / "child.py"
    script.write_text(CHILD.format(root=str(ROOT), tests=str(ROOT / "tests")))
    res = subprocess.run([sys.executable, str(script), kind, str(path), "7", "300"], capture_output=True, text=True,
                         timeout=240, env={**os.environ, "CUDA_VISIBLE_DEVICES": ""})
    assert res.returncode == 0, res.stderr[-2000:]
    ok, failed = map(int, res.stdout.split())
    assert ok + failed == 300 and failed > 0
