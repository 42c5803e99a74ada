"""ctypes binding of ``libmpm_gb300.so`` (the C ABI declared in include/mpm_gb300.h).

The library is built in-tree by :mod:`mpm_gb300.build`.  There is no fallback:
if the library cannot be loaded, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmpm_gb300.so")

MPM_MAX_MATERIALS = 16
STATUS_NAMES = {0: "MPM_OK", 1: "MPM_ERR_INVALID", 2: "MPM_ERR_CUDA", 3: "MPM_ERR_STATE", 4: "MPM_ERR_TIMEOUT",
                5: "MPM_ERR_NOMEM", 6: "MPM_ERR_UNSUPPORTED", 7: "MPM_ERR_IO"}


class MpmParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_float),
        ("N", ctypes.c_uint32),
        ("gravity", ctypes.c_float),
        ("boundary_mode", ctypes.c_int32),
        ("boundary_cells", ctypes.c_int32),
        ("g2p_guard", ctypes.c_int32),
        ("sort_interval", ctypes.c_int32),
        ("check_finite", ctypes.c_int32),
    ]


class MpmMaterial(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("particle_volume", ctypes.c_float),
        ("density", ctypes.c_float),
        ("E", ctypes.c_float),
        ("nu", ctypes.c_float),
        ("hardening", ctypes.c_float),
        ("clamp_lo", ctypes.c_float),
        ("clamp_hi", ctypes.c_float),
        ("bulk", ctypes.c_float),
    ]


class MpmScene(ctypes.Structure):
    _fields_ = [("params", MpmParams), ("material", MpmMaterial), ("count", ctypes.c_int64)]


SHAPE_BOX, SHAPE_SPHERE, SHAPE_MESH = 0, 1, 2
INSIDE_RAY_PARITY, INSIDE_WINDING = 0, 1


class MpmObject(ctypes.Structure):
    _fields_ = [
        ("shape", ctypes.c_int32),
        ("material", ctypes.c_int32),
        ("size", ctypes.c_float),
        ("position", ctypes.c_float * 3),
        ("velocity", ctypes.c_float * 3),
        ("box_extent", ctypes.c_float * 3),
        ("lifetime_begin", ctypes.c_double),
        ("lifetime_end", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("vertices", ctypes.c_void_p),
        ("n_vertices", ctypes.c_int64),
        ("triangles", ctypes.c_void_p),
        ("n_triangles", ctypes.c_int64),
        ("inside_test", ctypes.c_int32),
    ]


TILE_4x4x6, TILE_4x4x4, TILE_4x6x6 = 1, 2, 3
TUNE_SORT_INTERVAL, TUNE_IGNORE_CACHE = 1, 2


class MpmTuning(ctypes.Structure):
    _fields_ = [
        ("steps_per_warp", ctypes.c_int32),
        ("warps_per_cta", ctypes.c_int32),
        ("tile_box", ctypes.c_int32),
        ("sort_interval", ctypes.c_int32),
        ("us_per_substep", ctypes.c_double),
        ("from_cache", ctypes.c_int32),
        ("candidates", ctypes.c_int32),
    ]


# (name, restype, argtypes) for every entry point of include/mpm_gb300.h
P = ctypes.c_void_p
I32, I64 = ctypes.c_int32, ctypes.c_int64
SIGNATURES = [
    ("mpm_create", I32, [ctypes.POINTER(MpmParams), ctypes.POINTER(P)]),
    ("mpm_destroy", I32, [P]),
    ("mpm_set_stream", I32, [P, P]),
    ("mpm_set_params", I32, [P, ctypes.POINTER(MpmParams)]),
    ("mpm_set_materials", I32, [P, ctypes.POINTER(MpmMaterial), I32]),
    ("mpm_upload_soa", I32, [P, I64, P, P, P, P, P, P]),
    ("mpm_upload_aos", I32, [P, P, I64]),
    ("mpm_substep", I32, [P, I32]),
    ("mpm_sync", I32, [P]),
    ("mpm_download_soa", I32, [P, P, P, P, P, P, P]),
    ("mpm_download_aos", I32, [P, P]),
    ("mpm_get_grid", I32, [P, I32, P]),
    ("mpm_sort", I32, [P]),
    ("mpm_check_wait_timeout", I32, [P, I32]),
    ("mpm_add_object", I32, [P, ctypes.POINTER(MpmObject), ctypes.POINTER(I64)]),
    ("mpm_time", ctypes.c_double, [P]),
    ("mpm_object_count", I32, [P]),
    ("mpm_surface_distance", I32, [P, I32, I32, P]),
    ("mpm_surface_mesh", I32, [P, I32, I32, P, I64, ctypes.POINTER(I64)]),
    ("mpm_surface_mesh_device", I32, [P, I32, I32, ctypes.POINTER(P), ctypes.POINTER(I64)]),
    ("mpm_surface_mesh_indexed", I32, [P, I32, I32, P, I64, P, I64, ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    ("mpm_surface_mesh_indexed_device", I32, [P, I32, I32, ctypes.POINTER(P), ctypes.POINTER(P),
                                               ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    ("mpm_surface_table", I32, [P, P]),
    ("mpm_surface_smooth", I32, [P, P, I64, P, I64, ctypes.POINTER(I32)]),
    ("mpm_surface_smooth_device", I32, [P, P, I64, P, I64, ctypes.POINTER(I32)]),
    ("mpm_surface_distance_device", I32, [P, I32, I32, ctypes.POINTER(P)]),
    ("mpm_export_particles", I32, [P, I32, ctypes.c_float, ctypes.POINTER(I64)]),
    ("mpm_export_wait", I32, [P, I32, ctypes.POINTER(P), ctypes.POINTER(I64)]),
    ("mpm_write_bgeo", I32, [ctypes.c_char_p, P, I64]),
    ("mpm_bgeo_header", I64, [I64, P, I64]),
    ("mpm_render_positions_device", I32, [P, ctypes.POINTER(P)]),
    ("mpm_render_positions", I32, [P, P]),
    ("mpm_render_points", I32, [P, I32, I32, ctypes.c_float, P, P, P]),
    ("mpm_seed_object", I32, [ctypes.POINTER(MpmObject), ctypes.c_uint32, P, I64, ctypes.POINTER(I64)]),
    ("mpm_particle_count", I64, [P]),
    ("mpm_substep_count", I64, [P]),
    ("mpm_last_error", I32, [P, ctypes.c_char_p, ctypes.c_size_t]),
    ("mpm_launch_count", I64, [P]),
    ("mpm_set_tuning", I32, [P, I32, I32, I32]),
    ("mpm_substep_many", I32, [ctypes.POINTER(P), I32, I32]),
    ("mpm_autotune", I32, [P, ctypes.c_char_p, I32, I32, ctypes.POINTER(MpmTuning)]),
    ("mpm_get_tuning", I32, [P, ctypes.POINTER(MpmTuning)]),
    ("mpm_material_kind_available", I32, [I32]),
    ("mpm_batch_create", I32, [ctypes.POINTER(MpmScene), I32, I32, ctypes.POINTER(P)]),
    ("mpm_batch_destroy", I32, [P]),
    ("mpm_batch_set_stream", I32, [P, P]),
    ("mpm_batch_upload_soa", I32, [P, P, P, P, P, P]),
    ("mpm_batch_substep", I32, [P, I32]),
    ("mpm_batch_substep_graph", I32, [P, I32]),
    ("mpm_batch_sync", I32, [P]),
    ("mpm_batch_download_soa", I32, [P, P, P, P, P, P]),
    ("mpm_batch_particle_count", I64, [P]),
    ("mpm_batch_launch_count", I64, [P]),
    ("mpm_batch_last_error", I32, [P, ctypes.c_char_p, ctypes.c_size_t]),
    ("mpm_batch_set_steps_per_warp", I32, [P, I32]),
    ("mpm_batch_set_sort_interval", I32, [P, I32]),
    ("mpm_batch_get_tuning", I32, [P, ctypes.POINTER(MpmTuning)]),
    ("mpm_batch_autotune", I32, [P, ctypes.c_char_p, I32, I32, ctypes.POINTER(MpmTuning)]),
    ("mpm_diff_create", I32, [ctypes.POINTER(MpmParams), ctypes.POINTER(MpmMaterial), I64, I32, I32,
                              ctypes.POINTER(P)]),
    ("mpm_diff_destroy", I32, [P]),
    ("mpm_diff_set_material", I32, [P, ctypes.POINTER(MpmMaterial)]),
    ("mpm_diff_forward", I32, [P, P, P, P, P, P, I32, P, P]),
    ("mpm_diff_backward", I32, [P, P, P, P, P, P, P, P]),
    ("mpm_substep_noalloc", I32, [ctypes.POINTER(MpmParams), ctypes.POINTER(MpmMaterial), I32, P, I64, P, I64, I32,
                                  P]),
    ("mpm_noalloc_status", I32, [P]),
    ("mpm_noalloc_check_wait_timeout", I32, [I32, P]),
]

_lib = None


class MpmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


def load_library(path: str) -> ctypes.CDLL:
    """A build of the library at `path` (e.g. one with compiled-in material models from
    build.build_with_materials) with the entry points' signatures set."""
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing; run mpm_gb300.build.build() (needs nvcc)")
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib() -> ctypes.CDLL:
    """Load the CUDA library (raises if it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is None:
        _lib = load_library(LIB_PATH)
    return _lib


# the library each live context was created by (contexts of a build with compiled-in
# materials report their errors through that build)
_owner = {}


def register_context(ctx, L) -> None:
    _owner[ctx.value] = L


def forget_context(ctx) -> None:
    _owner.pop(ctx.value, None)


def check(code: int, ctx=None) -> None:
    if code != 0:
        msg = ""
        if ctx:
            buf = ctypes.create_string_buffer(512)
            (_owner.get(getattr(ctx, "value", None)) or lib()).mpm_last_error(ctx, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise MpmError(code, msg)
