"""CPU checks of the C ABI boundary: the library builds and loads without a GPU,
exports every entry point include/gbrt.h declares, and its ctypes mirror has
the C compiler's struct layout."""
import ctypes
import os
import re
import subprocess

import pytest

from renderer_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbrt.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbrt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gbrt_render" in names and "gbrt_trace_closest" in names
    assert set(names) == {n for n, _, _ in _abi.SIGNATURES}


def test_library_loads_and_exports_every_symbol(gbrt_built):
    lib = ctypes.CDLL(gbrt_built)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.gbrt_abi_version.restype = ctypes.c_int32
    assert lib.gbrt_abi_version() == 1


def test_exports_are_c_symbols(gbrt_built):
    out = subprocess.run(["nm", "-D", "--defined-only", gbrt_built], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gbrt_[a-z0-9_]+)\b", out))
    assert set(declared_functions()) <= exported


def test_struct_layout_matches_c(tmp_path):
    structs = ["gbrt_material", "gbrt_quad", "gbrt_sphere", "gbrt_plane", "gbrt_light", "gbrt_env_map",
               "gbrt_scene_desc", "gbrt_camera", "gbrt_render_params", "gbrt_stats", "gbrt_ray", "gbrt_hit",
               "gbrt_guide_params", "gbrt_guide_stats", "gbrt_texture", "gbrt_csg_node", "gbrt_batch_job",
               "gbrt_batch_stats", "gbrt_mlt_params", "gbrt_erpt_params", "gbrt_chain_stats",
               "gbrt_mesh", "gbrt_instance", "gbrt_batch_schedule"]
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "gbrt.h"\nint main(void){\n' +
                   "".join('printf("%%zu\\n", sizeof(%s));\n' % s for s in structs) + "return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    mirror = [_abi.Material, _abi.Quad, _abi.Sphere, _abi.Plane, _abi.Light, _abi.EnvMap, _abi.SceneDesc,
              _abi.Camera, _abi.RenderParams, _abi.Stats, _abi.Ray, _abi.Hit, _abi.GuideParams, _abi.GuideStats,
              _abi.Texture, _abi.CsgNode, _abi.BatchJob, _abi.BatchStats,
              _abi.MltParams, _abi.ErptParams, _abi.ChainStats, _abi.Mesh, _abi.Instance, _abi.BatchSchedule]
    assert sizes == [ctypes.sizeof(m) for m in mirror]
    assert ctypes.sizeof(_abi.Ray) == 32 and ctypes.sizeof(_abi.Hit) == 16


def test_errors_without_device_are_reported_not_raised(gbrt_built):
    """With no usable device, context creation fails with a status and a message."""
    import renderer_gb300 as rg
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    lib = rg.lib()
    h = ctypes.c_void_p()
    st = lib.gbrt_ctx_create(0, ctypes.byref(h))
    assert st == _abi.ERR_CUDA
    assert b"no CUDA device" in lib.gbrt_last_error(None)
    assert lib.gbrt_scene_create(None, None, None) == _abi.ERR_INVALID_ARG
