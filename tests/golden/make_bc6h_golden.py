"""Writes tests/golden/bc6h_texture_unit.json: seeded BC6H blocks of every
mode (and the four reserved mode values) with the binary16 texels the GPU's
texture unit decodes from them, as UF16 and as SF16.

Needs a CUDA GPU with BC6H texture support and nvcc: it builds
tests/bc_hw.cu (a block-compressed CUDA array read through a point-sampled
texture object) and runs it on the blocks.  The fixture pins the BC6H
oracle (oracle/texture.c) in the CPU tests.

    python tests/golden/make_bc6h_golden.py
"""
import base64
import json
import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# every 5-bit mode field value the format defines, then the reserved ones
MODES = [0x00, 0x01, 0x02, 0x06, 0x0A, 0x0E, 0x12, 0x16, 0x1A, 0x1E, 0x03, 0x07, 0x0B, 0x0F,
         0x13, 0x17, 0x1B, 0x1F]
PER_MODE = 8          # seeded random blocks per mode value
BLOCKS_PER_ROW = 32


def blocks() -> np.ndarray:
    rng = np.random.default_rng(61)
    out = []
    for m in MODES:
        mode_bits = 2 if m < 2 else 5
        for _ in range(PER_MODE):
            v = int.from_bytes(rng.integers(0, 256, 16, dtype=np.uint8).tobytes(), "little")
            out.append(((v & ~((1 << mode_bits) - 1)) | m).to_bytes(16, "little"))
        # every bit set beside the mode: the largest endpoints and deltas
        out.append((((1 << 128) - 1) & ~((1 << mode_bits) - 1) | m).to_bytes(16, "little"))
    out += [bytes(16)] * (-len(out) % BLOCKS_PER_ROW)
    return np.frombuffer(b"".join(out), np.uint8)


def main() -> None:
    data = blocks()
    w = BLOCKS_PER_ROW * 4
    h = data.size // 16 // BLOCKS_PER_ROW * 4
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    result = {"width": w, "height": h, "blocks": base64.b64encode(data.tobytes()).decode()}
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        exe = tmp / "bc_hw"
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", str(exe),
                        str(HERE.parent / "bc_hw.cu")], check=True)
        (tmp / "blocks.bin").write_bytes(data.tobytes())
        for fmt, key in ((9, "uf16"), (10, "sf16")):
            subprocess.run([str(exe), str(fmt), str(tmp / "blocks.bin"), str(tmp / "out.bin"), str(w), str(h)],
                           check=True)
            texels = np.fromfile(tmp / "out.bin", np.float32).reshape(h, w, 4)
            assert (texels[..., 3] == 1.0).all()
            half = texels[..., :3].astype(np.float16).view(np.uint16)  # exact: the values are binary16
            result[key] = base64.b64encode(np.ascontiguousarray(half).tobytes()).decode()
    (HERE / "bc6h_texture_unit.json").write_text(json.dumps(result, indent=0) + "\n")
    print(f"{data.size // 16} blocks, {w}x{h} texels")


if __name__ == "__main__":
    main()
