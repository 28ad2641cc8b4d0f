"""GB300-native (sm_103a) meshlet visibility-buffer path of vk_gltf_viewer.

The product is libvkgv.so (C ABI in include/vkgv.h); this package holds its
in-tree build, the ctypes mirror of the ABI, the host-side scene assembly and
the `Renderer` operator interface used by the tests and the benchmark.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "build", "scene", "renderer"]
