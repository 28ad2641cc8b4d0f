"""CPU checks of the drop-in boundary: the library builds for sm_103a, loads,
exports every function include/vkgv.h declares, and its structs match the
reference's scalar GLSL layouts byte for byte (mesh_common.h.glsl:20-126,
visbuffer.h.glsl:20-56).  No compute call is made (no GPU here)."""
import ctypes as C
import subprocess
import textwrap

import pytest

from vk_gltf_viewer_gb300 import abi


def test_library_exports_every_declared_symbol(built):
    lib = abi.load()
    names = abi.declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_string(built):
    assert b"sm_103a" in abi.load().vkgv_version()


@pytest.mark.parametrize("name,size", sorted(abi.EXPECTED_SIZES.items()))
def test_ctypes_struct_sizes(name, size):
    assert C.sizeof(getattr(abi, name)) == size


def test_c_layout_matches_ctypes(tmp_path):
    """Compiles a probe against include/vkgv.h with gcc and compares every
    field offset with the ctypes mirror."""
    structs = {
        "vkgv_meshlet": abi.Meshlet, "vkgv_vertex": abi.Vertex, "vkgv_meshlet_draw": abi.MeshletDraw,
        "vkgv_primitive": abi.Primitive, "vkgv_material": abi.Material, "vkgv_camera": abi.Camera,
        "vkgv_texture": abi.Texture, "vkgv_pyramid": abi.Pyramid, "vkgv_scene": abi.Scene, "vkgv_view": abi.View,
        "vkgv_config": abi.Config, "vkgv_mesh_info": abi.MeshInfo, "vkgv_meshlet_cone": abi.MeshletCone,
        "vkgv_node": abi.Node, "vkgv_anim_sampler": abi.AnimSampler, "vkgv_anim_channel": abi.AnimChannel,
        "vkgv_world_desc": abi.WorldDesc, "vkgv_gltf_info": abi.GltfInfo, "vkgv_gltf_primitive": abi.GltfPrimitive,
        "vkgv_gltf_image": abi.GltfImage, "vkgv_dds_info": abi.DdsInfo, "vkgv_jpeg_info": abi.JpegInfo,
    }
    lines = []
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} @sizeof %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    src = tmp_path / "probe.c"
    src.write_text(textwrap.dedent("""
        #include <stdio.h>
        #include <stddef.h>
        #include "vkgv.h"
        int main(void) {
        %s
        return 0; }
    """) % "\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", str(abi.ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, cls in structs.items():
        assert got[(cname, "@sizeof")] == C.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])


def test_oracle_layouts_match(built):
    """The oracle's own restatement of the layouts has the same sizes."""
    from oracle import binding  # noqa: F401  (built fixture compiled it)
    src = abi.ROOT / "oracle" / "oracle.h"
    probe = abi.ROOT / "oracle" / "_build" / "probe_sizes.c"
    probe.write_text('#include <stdio.h>\n#include "oracle.h"\nint main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",'
                     'sizeof(orc_meshlet), sizeof(orc_vertex), sizeof(orc_draw), sizeof(orc_material),'
                     'sizeof(orc_camera), sizeof(orc_node), sizeof(orc_anim_sampler), sizeof(orc_anim_channel),'
                     'sizeof(orc_world));return 0;}\n')
    exe = probe.with_suffix("")
    subprocess.run(["gcc", "-I", str(src.parent), str(probe), "-o", str(exe)], check=True)
    sizes = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    assert sizes == [36, 24, 12, 48, 352, 52, 32, 16, 96]


def test_pyramid_layout_host_helper(built):
    lib = abi.load()
    lv, fl = C.c_uint32(), C.c_uint64()
    assert lib.vkgv_pyramid_layout(1920, 1080, C.byref(lv), C.byref(fl)) == abi.OK
    assert lv.value == 10
    # mips 960x540, 480x270, ..., 1x1 (the last with a clamped height)
    exp = sum(max(1, 960 >> k) * max(1, 540 >> k) for k in range(10))
    assert fl.value == exp
    assert lib.vkgv_pyramid_layout(0, 5, C.byref(lv), C.byref(fl)) == abi.INVALID_ARG
    assert lib.vkgv_pyramid_layout(9000, 5, C.byref(lv), C.byref(fl)) == abi.INVALID_ARG


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    rc = abi.load().vkgv_create(None, C.byref(ctx))
    assert rc == abi.CUDA_ERROR and not ctx.value
