"""The C ABI: struct layouts against the C compiler, and every symbol of
include/gammaray.h exported by both libraries (loaded, not called: no GPU needed)."""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import pytest

from gammaray_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gammaray.h")

STRUCTS = {
    "gr_material_desc": _abi.MaterialDesc,
    "gr_prim_desc": _abi.PrimDesc,
    "gr_scene_desc": _abi.SceneDesc,
    "gr_scene_info": _abi.SceneInfo,
    "gr_camera": _abi.CameraDesc,
    "gr_render_params": _abi.RenderParams,
    "gr_render_stats": _abi.RenderStats,
    "gr_hit": _abi.Hit,
    "gr_light_sample": _abi.LightSampleOut,
    "gr_frame": _abi.Frame,
    "gr_bsdf_sample": _abi.BsdfSample,
    "gr_job": _abi.Job,
    "gr_batch_options": _abi.BatchOptions,
    "gr_server_options": _abi.ServerOptions,
    "gr_server_info": _abi.ServerInfo,
    "gr_request": _abi.Request,
    "gr_request_status": _abi.RequestStatus,
}


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(gr_\w+)\(", text, re.M)))


def test_header_functions_have_signatures():
    names = header_functions()
    assert len(names) > 30
    missing = [n for n in names if n not in _abi.SIGNATURES]
    assert not missing, missing


def test_struct_layout_matches_c(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gammaray.h"', "int main(void){"]
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split(
        "\n") if l)
    for cname, cls in STRUCTS.items():
        assert int(out[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"


def test_oracle_exports_every_symbol(oracle):
    for name in header_functions():
        if name in _abi.GPU_ONLY:
            continue
        assert hasattr(oracle.dll, name), name
    assert oracle.backend == "oracle-cpu"
    assert oracle.gr_abi_version() == 1


def _gpu_lib_path():
    import gammaray_gb300

    if not os.path.exists(gammaray_gb300.LIB_PATH):
        try:
            from gammaray_gb300 import build

            build.build()
        except Exception as e:  # no nvcc on this machine
            pytest.skip(f"cannot build the CUDA library here: {e}")
    return gammaray_gb300.LIB_PATH


def test_gpu_library_loads_and_exports_every_symbol():
    lib = C.CDLL(_gpu_lib_path())  # loading needs no GPU
    for name in header_functions():
        assert hasattr(lib, name), name
    lib.gr_backend_name.restype = C.c_char_p
    assert lib.gr_backend_name() == b"cuda-sm_103a"


def test_defaults_agree(oracle):
    gpu = _abi.Lib(_gpu_lib_path())
    for integ in (0, 1, 2):
        a, b = _abi.RenderParams(), _abi.RenderParams()
        oracle.gr_render_params_default(integ, C.byref(a))
        gpu.gr_render_params_default(integ, C.byref(b))
        assert bytes(a) == bytes(b)
    a, b = _abi.MaterialDesc(), _abi.MaterialDesc()
    oracle.gr_material_disney_defaults(C.byref(a))
    gpu.gr_material_disney_defaults(C.byref(b))
    assert bytes(a) == bytes(b)


def test_errors_are_reported_not_raised(oracle):
    with pytest.raises(_abi.GrError) as e:
        oracle.call("gr_film_create", 0, 10, C.byref(C.c_void_p()))
    assert e.value.status == 1
    assert "film size" in str(e.value)
