"""Writes tests/golden/zstd_frames.json: Zstandard frames made by libzstd
(through pyarrow's zstd codec) from seeded inputs of different kinds, sizes
and compression levels, with the SHA-256 of each input, so that the
library's decoder is checked against real encoder output also where pyarrow
is absent.  Run: python tests/golden/make_zstd_vectors.py"""
import base64
import hashlib
import json
from pathlib import Path

import numpy as np


def inputs():
    rng = np.random.default_rng(2024)
    yield "zeros", bytes(70000)
    yield "ramp", bytes(range(256)) * 300
    yield "text", b"the quick brown fox jumps over the lazy dog " * 1500
    # more than one 128 KiB block, with matches across block boundaries
    chunk = rng.integers(0, 256, 2048, dtype=np.uint8)
    yield "multi_block", np.concatenate([np.roll(chunk, int(k)) for k in rng.integers(0, 2048, 150)]).tobytes()
    yield "random", rng.integers(0, 256, 1500, dtype=np.uint8).tobytes()
    yield "low_entropy", rng.integers(0, 4, 6000, dtype=np.uint8).tobytes()
    yield "runs", b"".join(rng.integers(0, 256, int(k), dtype=np.uint8).tobytes() * int(r)
                           for k, r in zip(rng.integers(1, 40, 200), rng.integers(1, 6, 200)))
    yield "bc1_blocks", np.tile(rng.integers(0, 256, 8 * 64, dtype=np.uint8), 300).tobytes()
    yield "tiny", b"abc"
    yield "empty", b""


def main():
    import pyarrow as pa

    cases = []
    for name, data in inputs():
        for level in (1, 19, -5):
            frame = pa.Codec("zstd", compression_level=level).compress(data, asbytes=True)
            cases.append({"name": name, "level": level, "size": len(data),
                          "sha256": hashlib.sha256(data).hexdigest(),
                          "frame": base64.b64encode(frame).decode()})
    path = Path(__file__).resolve().parent / "zstd_frames.json"
    path.write_text(json.dumps({"source": "libzstd via pyarrow " + pa.__version__, "cases": cases}, indent=0) + "\n")
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(cases)} frames)")


if __name__ == "__main__":
    main()
