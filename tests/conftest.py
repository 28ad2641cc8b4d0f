import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds libvkgv.so and the oracle once per session."""
    from vk_gltf_viewer_gb300 import build as vbuild
    from oracle import binding

    vbuild.build()
    binding.build()
    binding.build_ref()
    binding.set_threads(min(8, os.cpu_count() or 1))
    return True


@pytest.fixture(scope="session")
def renderer(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vk_gltf_viewer_gb300.renderer import Renderer

    r = Renderer(0)
    yield r
    r.close()
