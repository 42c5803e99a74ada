"""Golden distance fields from the reference's own include/mesh_builder.h.

``make(lib_path)`` drives ``oracle/_ref/libref_mesh.so`` (the header's
fillVoxelGrid_distance with MeshBuilder::computeMesh's arguments, compiled for the host)
over seeded particle sets and returns arrays for ``ref_mesh.npz``.  Called by
make_golden.py here, where the reference checkout exists; the tests only read the .npz.

Particles are drawn uniformly in [-r voxel_dx, 1 + 2 voxel_dx)^3, so the set covers
nodes clipped at both faces of the grid (a particle more than the cutoff below the
origin would make the reference's unsigned loop bound wrap, so none is drawn there).

Mesh cases (``mesh_<case>``) run MeshBuilder::computeMesh itself (the header's own code
with libigl's marching cubes from the reference's vendored include/igl/copyleft/) on a
ball, a sparse cloud (many ambiguous cube faces) and a cluster cut by the grid's corner,
and store the V and F it hands to igl::writeOBJ; the largest (the reference's default
grid, G = 250 with radius 5) stores the sha256 of V and the face count only.

Cases ``<case>_x`` (particles), ``<case>_params`` (N, G, radius), ``<case>_voxel_dx``
and either ``<case>_field`` (G^3 floats; the first case only, to keep the fixture small)
or ``<case>_sha256`` of the field's bytes (the others, among them the reference's
default mesh grid, G = 250 with radius 5).
"""
import ctypes
import hashlib

import numpy as np

CASES = (  # name, N, G, radius, particles, store the field
    ("sparse_r1", 64, 32, 1, 300, True),
    ("mid_r2", 64, 40, 2, 600, False),
    ("wide_r5", 100, 48, 5, 200, False),
    ("odd_r3", 17, 33, 3, 400, False),
    ("default_G250_r5", 32, 250, 5, 2000, False),
)


MESH_CASES = (  # name, N, G, radius, kind, particles, store V and F
    ("ball_G40_r2", 32, 40, 2, "ball", 3000, True),
    ("cloud_G16_r1", 32, 16, 1, "cloud", 120, True),
    ("corner_G20_r3", 32, 20, 3, "corner", 400, True),
    ("default_G250_r5", 60, 250, 5, "ball", 4000, False),
)


def _particles(rng, kind, n):
    if kind == "ball":
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        return (0.5 + u * (0.25 * rng.random(n) ** (1 / 3))[:, None]).astype(np.float32)
    if kind == "corner":
        return rng.uniform(0.0, 0.15, (n, 3)).astype(np.float32)
    return rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)


def load(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.ref_voxel_dx.restype = ctypes.c_double
    lib.ref_voxel_dx.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    I64 = ctypes.c_int64
    lib.ref_compute_mesh.restype = ctypes.c_int
    lib.ref_compute_mesh.argtypes = [ctypes.c_void_p, I64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_void_p, I64, ctypes.c_void_p, I64, ctypes.c_void_p, ctypes.c_void_p]
    lib.ref_distance_field.restype = ctypes.c_int
    lib.ref_distance_field.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_double, ctypes.c_void_p]
    return lib


def field_sha256(field):
    return hashlib.sha256(np.ascontiguousarray(field, np.float32).tobytes()).hexdigest()


def compute_mesh(lib, x, N, G, r):
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    assert lib.ref_compute_mesh(x.ctypes.data, len(x), N, G, r, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nf)) == 0
    V = np.empty((max(nv.value, 1), 3), np.float64)
    F = np.empty((max(nf.value, 1), 3), np.int32)
    lib.ref_compute_mesh(x.ctypes.data, len(x), N, G, r, V.ctypes.data, nv.value, F.ctypes.data, nf.value,
                         ctypes.byref(nv), ctypes.byref(nf))
    return V[:nv.value], F[:nf.value]


def make(lib_path):
    lib = load(lib_path)
    rng = np.random.default_rng(77)
    out = {}
    for name, N, G, r, n, store in CASES:
        vdx = lib.ref_voxel_dx(N, G)
        x = rng.uniform(-r * vdx, 1.0 + 2 * vdx, (n, 3)).astype(np.float32)
        f = np.empty((G, G, G), np.float32)
        assert lib.ref_distance_field(x.ctypes.data, n, G, r, vdx, f.ctypes.data) == 0
        out[name + "_x"] = x
        out[name + "_params"] = np.array([N, G, r], np.int64)
        out[name + "_voxel_dx"] = np.array(vdx, np.float64)
        if store:
            out[name + "_field"] = f
        else:
            out[name + "_sha256"] = np.array(field_sha256(f))
    rng = np.random.default_rng(91)
    for name, N, G, r, kind, n, store in MESH_CASES:
        x = _particles(rng, kind, n)
        V, F = compute_mesh(lib, x, N, G, r)
        key = "mesh_" + name
        out[key + "_x"] = x
        out[key + "_params"] = np.array([N, G, r], np.int64)
        out[key + "_nf"] = np.array(len(F), np.int64)
        if store:
            out[key + "_V"] = V
            out[key + "_F"] = F
        else:
            out[key + "_Vsha256"] = np.array(hashlib.sha256(np.ascontiguousarray(V).tobytes()).hexdigest())
            out[key + "_nv"] = np.array(len(V), np.int64)
    return out
