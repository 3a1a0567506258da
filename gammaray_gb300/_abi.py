"""ctypes mirror of include/gammaray.h.

Both shared libraries that implement the header (the CUDA library in this package and
the CPU restatement under oracle/) are loaded through `Lib`, so host code and tests
drive either one with the same calls.  Struct layouts below must match the header
field for field; `tests/test_abi.py` checks their sizes against the C compiler.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

GR_OK = 0
STATUS_NAMES = {
    0: "GR_OK",
    1: "GR_ERR_INVALID_ARGUMENT",
    2: "GR_ERR_OUT_OF_MEMORY",
    3: "GR_ERR_CUDA",
    4: "GR_ERR_UNSUPPORTED",
    5: "GR_ERR_TIMEOUT",
    6: "GR_ERR_STACK_OVERFLOW",
    7: "GR_ERR_NOT_FOUND",
    8: "GR_ERR_BUSY",
    9: "GR_ERR_CANCELLED",
    10: "GR_ERR_INTERNAL",
}

MATERIAL_DISNEY, MATERIAL_DIFFUSE_LIGHT, MATERIAL_DIFFUSE, MATERIAL_MIRROR = 0, 1, 2, 3
PRIM_MESH, PRIM_SPHERE = 0, 1
INTEGRATOR_PATH_TRACER, INTEGRATOR_BDPT, INTEGRATOR_DISPLAY_COLOR = 0, 1, 2
NO_INDEX = 0xFFFFFFFF

LOBE_NONE, LOBE_DIFFUSE, LOBE_SPECULAR, LOBE_GLOSSY, LOBE_REFLECTION, LOBE_TRANSMISSION = 0, 1, 2, 4, 8, 16

F3 = C.c_float * 3


class GrError(RuntimeError):
    """A gr_status other than GR_OK, with the library's gr_last_error() text."""

    def __init__(self, status: int, message: str, call: str):
        self.status = status
        super().__init__(f"{call}: {STATUS_NAMES.get(status, status)}: {message}")


class MaterialDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("base_color", F3),
        ("roughness", C.c_float),
        ("anisotropic", C.c_float),
        ("ior", C.c_float),
        ("metallic", C.c_float),
        ("specular_trans", C.c_float),
        ("specular_tint", C.c_float),
        ("sheen", C.c_float),
        ("sheen_tint", C.c_float),
        ("clearcoat", C.c_float),
        ("clearcoat_gloss", C.c_float),
        ("incandescence", F3),
    ]


class PrimDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("material", C.c_uint32),
        ("vertices", C.POINTER(C.c_float)),
        ("num_vertices", C.c_uint32),
        ("tri_vertices", C.POINTER(C.c_uint32)),
        ("num_tris", C.c_uint32),
        ("normals", C.POINTER(C.c_float)),
        ("num_normals", C.c_uint32),
        ("tri_normals", C.POINTER(C.c_uint32)),
        ("uvs", C.POINTER(C.c_float)),
        ("num_uvs", C.c_uint32),
        ("tri_uvs", C.POINTER(C.c_uint32)),
        ("center", F3),
        ("radius", C.c_float),
    ]


class SceneDesc(C.Structure):
    _fields_ = [
        ("materials", C.POINTER(MaterialDesc)),
        ("num_materials", C.c_uint32),
        ("prims", C.POINTER(PrimDesc)),
        ("num_prims", C.c_uint32),
        ("environment", F3),
        ("bvh_width", C.c_uint32),
        ("leaf_size", C.c_uint32),
        ("build", C.c_uint32),
    ]


BUILD_HOST_SAH = 0
BUILD_DEVICE_LBVH = 1


class SceneInfo(C.Structure):
    _fields_ = [
        ("num_components", C.c_uint64),
        ("num_binary_nodes", C.c_uint64),
        ("num_wide_nodes", C.c_uint64),
        ("device_bytes", C.c_uint64),
        ("num_lights", C.c_uint32),
        ("bvh_width", C.c_uint32),
        ("build_seconds", C.c_double),
        ("tree_hash", C.c_uint64),
        ("stack_depth", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class CameraDesc(C.Structure):
    _fields_ = [
        ("focal_length", C.c_float),
        ("horizontal_aperture", C.c_float),
        ("vertical_aperture", C.c_float),
        ("f_stop", C.c_float),
        ("rotate", C.c_float * 4),
        ("translate", F3),
    ]


class RenderParams(C.Structure):
    _fields_ = [
        ("integrator", C.c_int32),
        ("spp", C.c_uint32),
        ("max_depth", C.c_uint32),
        ("rr_depth", C.c_uint32),
        ("rr_aggressive_depth", C.c_uint32),
        ("mis", C.c_uint32),
        ("light_tracing", C.c_uint32),
        ("first_pass", C.c_uint32),
        ("seed", C.c_uint64),
        ("flags", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


RENDER_COUNT_TRAVERSAL = 1
RENDER_TIME_KERNELS = 2


class RenderStats(C.Structure):
    _fields_ = [
        ("samples", C.c_uint64),
        ("extension_rays", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("node_visits", C.c_uint64),
        ("prim_tests", C.c_uint64),
        ("extend_launches", C.c_uint64),
        ("device_ms", C.c_double),
        ("extend_ms", C.c_double),
        ("shade_ms", C.c_double),
        ("raygen_ms", C.c_double),
        ("film_ms", C.c_double),
    ]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_int32), ("component", C.c_int32), ("u", C.c_float), ("v", C.c_float)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<i4"), ("component", "<i4"), ("u", "<f4"), ("v", "<f4")])


class LightSampleOut(C.Structure):
    _fields_ = [
        ("origin", F3),
        ("direction", F3),
        ("normal", F3),
        ("tangent", F3),
        ("binormal", F3),
        ("geom_normal", F3),
        ("prim", C.c_int32),
        ("point_pdf", C.c_float),
        ("dir_pdf", C.c_float),
    ]


LIGHT_SAMPLE_DTYPE = np.dtype(
    [
        ("origin", "<f4", 3),
        ("direction", "<f4", 3),
        ("normal", "<f4", 3),
        ("tangent", "<f4", 3),
        ("binormal", "<f4", 3),
        ("geom_normal", "<f4", 3),
        ("prim", "<i4"),
        ("point_pdf", "<f4"),
        ("dir_pdf", "<f4"),
    ]
)


class Frame(C.Structure):
    _fields_ = [("normal", F3), ("tangent", F3), ("binormal", F3), ("geom_normal", F3)]


FRAME_DTYPE = np.dtype([("normal", "<f4", 3), ("tangent", "<f4", 3), ("binormal", "<f4", 3), ("geom_normal", "<f4", 3)])


class BsdfSample(C.Structure):
    _fields_ = [
        ("emission", F3),
        ("radiance", F3),
        ("outgoing", F3),
        ("pdf", C.c_float),
        ("kind", C.c_uint32),
    ]


BSDF_SAMPLE_DTYPE = np.dtype(
    [("emission", "<f4", 3), ("radiance", "<f4", 3), ("outgoing", "<f4", 3), ("pdf", "<f4"), ("kind", "<u4")]
)


class Job(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p),
        ("camera", CameraDesc),
        ("params", RenderParams),
        ("film", C.c_void_p),
    ]


class BatchOptions(C.Structure):
    _fields_ = [
        ("path_capacity", C.c_uint32),
        ("block_size", C.c_uint32),
        ("use_graph", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class ServerOptions(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_uint64),
        ("max_active", C.c_uint32),
        ("path_capacity", C.c_uint32),
        ("bvh_width", C.c_uint32),
        ("block_size", C.c_uint32),
        ("policy", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class ServerInfo(C.Structure):
    _fields_ = [
        ("queued", C.c_uint32),
        ("running", C.c_uint32),
        ("finished", C.c_uint32),
        ("engine_jobs", C.c_uint32),
        ("engine_units", C.c_uint64),
        ("resets", C.c_uint64),
        ("film_bytes", C.c_uint64),
        ("memory_budget_bytes", C.c_uint64),
    ]


SERVE_ARRIVAL_ORDER = 0
SERVE_SHORTEST_FIRST = 1


class Request(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p),
        ("camera", CameraDesc),
        ("params", RenderParams),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("target_rel_mse", C.c_float),
        ("reserved", C.c_uint32),
    ]


class RequestStatus(C.Structure):
    _fields_ = [
        ("state", C.c_int32),
        ("passes_done", C.c_uint32),
        ("submit_ms", C.c_double),
        ("start_ms", C.c_double),
        ("finish_ms", C.c_double),
        ("rel_mse", C.c_float),
        ("reserved", C.c_uint32),
    ]


# name -> (restype, argtypes); restype None = void.  Every symbol of include/gammaray.h.
_VP = C.c_void_p
_PF = C.POINTER(C.c_float)
SIGNATURES = {
    "gr_last_error": (C.c_char_p, []),
    "gr_abi_version": (C.c_int, []),
    "gr_backend_name": (C.c_char_p, []),
    "gr_material_disney_defaults": (None, [C.POINTER(MaterialDesc)]),
    "gr_scene_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(_VP)]),
    "gr_scene_destroy": (C.c_int, [_VP]),
    "gr_scene_plan": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(SceneInfo)]),
    "gr_scene_get_info": (C.c_int, [_VP, C.POINTER(SceneInfo)]),
    "gr_film_create": (C.c_int, [C.c_uint32, C.c_uint32, C.POINTER(_VP)]),
    "gr_film_destroy": (C.c_int, [_VP]),
    "gr_film_clear": (C.c_int, [_VP]),
    "gr_film_read": (C.c_int, [_VP, _PF, _PF]),
    "gr_film_resolve": (C.c_int, [_VP, _PF]),
    "gr_film_write_exr": (C.c_int, [_VP, C.c_char_p]),
    "gr_film_passes": (C.c_int, [_VP, C.POINTER(C.c_uint32)]),
    "gr_film_read_splat": (C.c_int, [_VP, _PF]),
    "gr_render_params_default": (None, [C.c_int32, C.POINTER(RenderParams)]),
    "gr_render": (C.c_int, [_VP, C.POINTER(CameraDesc), C.POINTER(RenderParams), _VP]),
    "gr_render_samples": (
        C.c_int,
        [_VP, C.POINTER(CameraDesc), C.POINTER(RenderParams), C.c_uint32, C.c_uint32, _PF],
    ),
    "gr_scene_last_stats": (C.c_int, [_VP, C.POINTER(RenderStats)]),
    "gr_render_static": (
        C.c_int,
        [_VP, C.POINTER(CameraDesc), C.POINTER(RenderParams), C.c_uint32, C.c_uint32, _VP, _VP],
    ),
    "gr_trace_rays": (C.c_int, [_VP, _PF, C.c_uint64, C.POINTER(Hit)]),
    "gr_trace_rays_dev": (C.c_int, [_VP, _VP, C.c_uint64, _VP, _VP]),
    "gr_intersect_naive": (C.c_int, [_VP, _PF, C.c_uint64, C.POINTER(Hit)]),
    "gr_visibility": (C.c_int, [_VP, _PF, C.c_uint64, C.POINTER(C.c_uint8)]),
    "gr_sample_light": (C.c_int, [_VP, _PF, C.c_uint64, C.POINTER(LightSampleOut)]),
    "gr_bsdf_eval": (
        C.c_int,
        [C.POINTER(MaterialDesc), C.c_uint64, C.POINTER(Frame), _PF, _PF, C.c_int32, _PF],
    ),
    "gr_bsdf_pdf": (C.c_int, [C.POINTER(MaterialDesc), C.c_uint64, C.POINTER(Frame), _PF, _PF, _PF]),
    "gr_bsdf_sample_batch": (
        C.c_int,
        [C.POINTER(MaterialDesc), C.c_uint64, C.POINTER(Frame), _PF, _PF, C.c_int32, C.POINTER(BsdfSample)],
    ),
    "gr_light_eval": (C.c_int, [C.POINTER(MaterialDesc), C.c_uint64, C.POINTER(Frame), _PF, _PF]),
    "gr_render_batch": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(BatchOptions)]),
    "gr_batch_autotune": (C.c_int, [C.POINTER(Job), C.c_uint32, C.POINTER(BatchOptions)]),
    "gr_batch_last_stats": (C.c_int, [C.POINTER(RenderStats)]),
    "gr_batch_release": (C.c_int, []),
    "gr_server_create": (C.c_int, [C.POINTER(ServerOptions), C.POINTER(_VP)]),
    "gr_server_destroy": (C.c_int, [_VP]),
    "gr_server_submit": (C.c_int, [_VP, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "gr_server_step": (C.c_int, [_VP, C.c_double]),
    "gr_server_poll": (C.c_int, [_VP, C.c_uint64, C.POINTER(RequestStatus)]),
    "gr_server_cancel": (C.c_int, [_VP, C.c_uint64]),
    "gr_server_take": (C.c_int, [_VP, C.c_uint64, _PF, _PF]),
    "gr_server_snapshot": (C.c_int, [_VP, C.c_uint64, _PF, _PF, C.POINTER(C.c_uint32)]),
    "gr_server_get_info": (C.c_int, [_VP, C.POINTER(ServerInfo)]),
}


# Entry points that only the CUDA library exports.
GPU_ONLY = {"gr_render_static"}


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def uptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class Lib:
    """One loaded implementation of include/gammaray.h."""

    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.path = path
        self.dll = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            if name in GPU_ONLY and not hasattr(self.dll, name):
                continue
            fn = getattr(self.dll, name)
            fn.restype = res
            fn.argtypes = args
        self.backend = self.dll.gr_backend_name().decode()

    def check(self, status: int, call: str):
        if status != GR_OK:
            raise GrError(status, self.dll.gr_last_error().decode(), call)

    def call(self, name: str, *args):
        self.check(getattr(self.dll, name)(*args), name)

    def __getattr__(self, name):
        if name.startswith("gr_"):
            return getattr(self.dll, name)
        raise AttributeError(name)
