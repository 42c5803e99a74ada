"""CPU oracle for the MLS-MPM substep — test infrastructure only.

This package is the checker for the CUDA path, never the product: only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (cpu_baseline and
``--impl reference``) may import it.  It wraps ``libmpm_oracle.so``, a C++
restatement of the reference substep (src/mpm.cu:14-178, 323-329 of
kekeblom/mpm) in FP32 and FP64, built by :func:`oracle.build.build_oracle`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libmpm_oracle.so")
MAX_MATERIALS = 16

MAT_SNOW, MAT_FIXED_COROTATED, MAT_JELLY, MAT_LIQUID = 0, 1, 2, 3
BOUNDARY_REF_FRACTION, BOUNDARY_STICKY_CELLS, BOUNDARY_SEPARATE_CELLS = 0, 1, 2


class OracleMaterial(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("particle_volume", ctypes.c_float),
        ("particle_mass", ctypes.c_float),
        ("mu0", ctypes.c_float),
        ("lambda0", ctypes.c_float),
        ("hardening", ctypes.c_float),
        ("clamp_lo", ctypes.c_float),
        ("clamp_hi", ctypes.c_float),
        ("bulk", ctypes.c_float),
    ]


class OracleConfig(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_float),
        ("N", ctypes.c_int),
        ("gravity", ctypes.c_float),
        ("boundary_mode", ctypes.c_int),
        ("boundary_cells", ctypes.c_int),
        ("g2p_guard", ctypes.c_int),
        ("nthreads", ctypes.c_int),
        ("n_materials", ctypes.c_int),
        ("materials", OracleMaterial * MAX_MATERIALS),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            from . import build as _b

            _b.build_oracle()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        for name in ("oracle_substep_f64", "oracle_substep_f32"):
            fn = getattr(L, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [P, ctypes.c_int64, P, P, P, P, P, P, ctypes.c_int, P, P]
        L.oracle_time_f32.restype = ctypes.c_double
        L.oracle_time_f32.argtypes = [P, ctypes.c_int64, P, P, P, P, P, P, ctypes.c_int]
        for name in ("oracle_svd_f32", "oracle_svd_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_int64, P, P, P, P]
        for name in ("oracle_polar_f32", "oracle_polar_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_int64, P, P, P]
        L.oracle_det_f32.restype = ctypes.c_float
        L.oracle_det_f32.argtypes = [P]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_seed_object.restype = ctypes.c_int64
        L.oracle_seed_object.argtypes = [ctypes.c_int, ctypes.c_float, P, P, ctypes.c_uint64, ctypes.c_uint32, P,
                                         ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int32, P, ctypes.c_int64]
        L.oracle_distance_field.restype = None
        L.oracle_distance_field.argtypes = [P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, P]
        L.oracle_surface_indexed.restype = None
        L.oracle_surface_indexed.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, P, ctypes.c_int64, P,
                                             ctypes.c_int64, P, P]
        L.oracle_surface_table.restype = None
        L.oracle_surface_table.argtypes = [P, P]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def make_config(params: dict, materials: list, nthreads: int = 0) -> OracleConfig:
    """Build the oracle config from the same dictionaries the product API takes.

    ``materials`` entries carry the derived float32 constants (see
    ``mpm_gb300.materials.derive``) so both sides see identical numbers."""
    cfg = OracleConfig()
    cfg.dt = float(params["dt"])
    cfg.N = int(params["N"])
    cfg.gravity = float(params.get("gravity", -9.81))
    cfg.boundary_mode = int(params.get("boundary_mode", BOUNDARY_REF_FRACTION))
    cfg.boundary_cells = int(params.get("boundary_cells", 3))
    cfg.g2p_guard = int(params.get("g2p_guard", 0))
    cfg.nthreads = int(nthreads)
    cfg.n_materials = len(materials)
    for i, m in enumerate(materials):
        om = cfg.materials[i]
        om.kind = int(m["kind"])
        om.particle_volume = float(m["particle_volume"])
        om.particle_mass = float(m["particle_mass"])
        om.mu0 = float(m["mu0"])
        om.lambda0 = float(m["lambda0"])
        om.hardening = float(m["hardening"])
        om.clamp_lo = float(m["clamp_lo"])
        om.clamp_hi = float(m["clamp_hi"])
        om.bulk = float(m["bulk"])
    return cfg


def substep(state: dict, params: dict, materials: list, nsteps: int = 1, dtype=np.float64,
            nthreads: int = 0, want_grids: bool = False):
    """Advance a copy of ``state`` by ``nsteps`` substeps on the CPU.

    ``state`` holds x (n,3), v (n,3), C (n,3,3), F (n,3,3), Jp (n,), mat (n,) u8.
    Returns (new_state, grid_p2g, grid_op) with grids shaped (N,N,N,4) when
    ``want_grids`` (the last substep's grid after P2G and after the grid op)."""
    L = lib()
    n = int(state["x"].shape[0])
    out = {k: np.ascontiguousarray(np.array(state[k], dtype=dtype)) for k in ("x", "v", "C", "F", "Jp")}
    mat = np.ascontiguousarray(np.asarray(state.get("mat", np.zeros(n, np.uint8)), dtype=np.uint8))
    cfg = make_config(params, materials, nthreads)
    N = cfg.N
    g1 = g2 = None
    if want_grids:
        g1 = np.zeros((N, N, N, 4), dtype=dtype)
        g2 = np.zeros((N, N, N, 4), dtype=dtype)
    fn = L.oracle_substep_f64 if dtype == np.float64 else L.oracle_substep_f32
    rc = fn(ctypes.byref(cfg), n, _ptr(out["x"]), _ptr(out["v"]), _ptr(out["C"]), _ptr(out["F"]),
            _ptr(out["Jp"]), _ptr(mat), int(nsteps), _ptr(g1), _ptr(g2))
    if rc != 0:
        raise RuntimeError(f"oracle substep failed with code {rc}")
    out["mat"] = mat
    return out, g1, g2


def time_f32(state: dict, params: dict, materials: list, nsteps: int, nthreads: int = 0) -> float:
    """Seconds for ``nsteps`` FP32 substeps of the restated reference on ``nthreads`` threads."""
    L = lib()
    n = int(state["x"].shape[0])
    arr = {k: np.ascontiguousarray(np.array(state[k], dtype=np.float32)) for k in ("x", "v", "C", "F", "Jp")}
    mat = np.ascontiguousarray(np.asarray(state.get("mat", np.zeros(n, np.uint8)), dtype=np.uint8))
    cfg = make_config(params, materials, nthreads)
    t = L.oracle_time_f32(ctypes.byref(cfg), n, _ptr(arr["x"]), _ptr(arr["v"]), _ptr(arr["C"]),
                          _ptr(arr["F"]), _ptr(arr["Jp"]), _ptr(mat), int(nsteps))
    if t < 0:
        raise RuntimeError("oracle timing run failed")
    return t


def svd(A: np.ndarray, dtype=np.float64):
    L = lib()
    A = np.ascontiguousarray(np.asarray(A, dtype=dtype).reshape(-1, 3, 3))
    n = A.shape[0]
    U = np.zeros_like(A)
    V = np.zeros_like(A)
    s = np.zeros((n, 3), dtype=dtype)
    fn = L.oracle_svd_f64 if dtype == np.float64 else L.oracle_svd_f32
    fn(n, _ptr(A), _ptr(U), _ptr(s), _ptr(V))
    return U, s, V


def polar(A: np.ndarray, dtype=np.float64):
    L = lib()
    A = np.ascontiguousarray(np.asarray(A, dtype=dtype).reshape(-1, 3, 3))
    R = np.zeros_like(A)
    S = np.zeros_like(A)
    fn = L.oracle_polar_f64 if dtype == np.float64 else L.oracle_polar_f32
    fn(A.shape[0], _ptr(A), _ptr(R), _ptr(S))
    return R, S


def det_f32(M: np.ndarray) -> float:
    M = np.ascontiguousarray(np.asarray(M, dtype=np.float32).reshape(9))
    return float(lib().oracle_det_f32(_ptr(M)))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def seed_object(shape: int, size: float, position, box_extent=(1.0, 1.0, 1.0), seed: int = 0, density: int = 1000,
                vertices=None, triangles=None, inside_test: int = 0) -> np.ndarray:
    """Positions (n, 3) float32 of the restated rejection sampler (oracle/seed_oracle.cpp)."""
    L = lib()
    pos = np.ascontiguousarray(np.asarray(position, np.float32).reshape(3))
    ext = np.ascontiguousarray(np.asarray(box_extent, np.float32).reshape(3))
    V = T = None
    nv = nt = 0
    if vertices is not None:
        V = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 3))
        T = np.ascontiguousarray(np.asarray(triangles, np.int32).reshape(-1, 3))
        nv, nt = V.shape[0], T.shape[0]
    args = (int(shape), float(size), _ptr(pos), _ptr(ext), int(seed) & 0xFFFFFFFFFFFFFFFF, int(density), _ptr(V),
            nv, _ptr(T), nt, int(inside_test))
    n = L.oracle_seed_object(*args, None, 0)
    if n < 0:
        raise ValueError("invalid object")
    x = np.empty((max(n, 1), 3), np.float32)
    L.oracle_seed_object(*args, _ptr(x), n)
    return x[:n]


def voxel_dx(N: int, dx: float, grid_side: int) -> float:
    """voxel_dx = N dx / grid_side with N dx in float (include/mesh_builder.h:172)."""
    return float(np.float32(np.float32(N) * np.float32(dx))) / float(grid_side)


def distance_field(x: np.ndarray, grid_side: int, radius: int, vdx: float) -> np.ndarray:
    """Distance field (G, G, G) float32 of oracle/surface_oracle.cpp."""
    X = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, 3))
    f = np.empty((grid_side,) * 3, np.float32)
    lib().oracle_distance_field(_ptr(X), X.shape[0], int(grid_side), int(radius), float(vdx), _ptr(f))
    return f


def surface_indexed(field: np.ndarray, radius: int, vdx: float):
    """Marching-cubes vertices (nv, 3) float64 and faces (nf, 3) int32 of the level set
    radius vdx - field = 0 (oracle/surface_oracle.cpp)."""
    f = np.ascontiguousarray(field, np.float32)
    G = f.shape[0]
    L = lib()
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    L.oracle_surface_indexed(_ptr(f), G, int(radius), float(vdx), None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nf))
    V = np.empty((max(nv.value, 1), 3), np.float64)
    F = np.empty((max(nf.value, 1), 3), np.int32)
    L.oracle_surface_indexed(_ptr(f), G, int(radius), float(vdx), _ptr(V), nv.value, _ptr(F), nf.value,
                             ctypes.byref(nv), ctypes.byref(nf))
    return V[:nv.value], F[:nf.value]


def surface_mesh(field: np.ndarray, radius: int, vdx: float) -> np.ndarray:
    """Triangles (T, 3, 3) float32: the faces' vertices rounded to float."""
    V, F = surface_indexed(field, radius, vdx)
    return V[F].astype(np.float32)


def surface_table():
    """The oracle's triangle table: counts (256,) and edge-slot triples (256, 30), -1 padded."""
    n = np.empty(256, np.int32)
    t = np.empty((256, 30), np.int32)
    lib().oracle_surface_table(_ptr(n), _ptr(t))
    return n, t
