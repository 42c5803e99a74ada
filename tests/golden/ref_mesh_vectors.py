"""Golden distance fields from the reference's own include/mesh_builder.h.

``make(lib_path)`` drives ``oracle/_ref/libref_mesh.so`` (the header's
fillVoxelGrid_distance with MeshBuilder::computeMesh's arguments, compiled for the host)
over seeded particle sets and returns arrays for ``ref_mesh.npz``.  Called by
make_golden.py here, where the reference checkout exists; the tests only read the .npz.

Particles are drawn uniformly in [-r voxel_dx, 1 + 2 voxel_dx)^3, so the set covers
nodes clipped at both faces of the grid (a particle more than the cutoff below the
origin would make the reference's unsigned loop bound wrap, so none is drawn there).

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


def load(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.ref_voxel_dx.restype = ctypes.c_double
    lib.ref_voxel_dx.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    lib.ref_distance_field.restype = ctypes.c_int
    lib.ref_distance_field.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_double, ctypes.c_void_p]
    return lib


def field_sha256(field):
    return hashlib.sha256(np.ascontiguousarray(field, np.float32).tobytes()).hexdigest()


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
    return out
