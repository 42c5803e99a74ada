"""Golden substep vectors from the reference's own policy headers.

``make(lib_path)`` drives ``oracle/_ref/libref_substep.so`` (the reference's
TransferScheme.h / MaterialModel.cuh / InterpolationKernel.cuh / linalg.cu compiled
for the host, under the loop of src/mpm.cu:14-178) over small seeded particle states
and returns arrays for ``ref_substep.npz``.  Called by make_golden.py here, where
the reference checkout exists; the tests only read the .npz.

Cases (all MMSnow, the only material the reference binds, include/mpm.cuh:25):
  elastic1  N=16, 2000 particles, 1 substep, hardening 0, clamps [0, 1e30]
  elastic4  the same state, 4 substeps
  snow1     N=16, 2000 particles, 1 substep, snowman parameters (plasticity active)
  snow3     the same state, 3 substeps
  mixed2    N=24, 3000 particles, two materials (snow, elastic), 2 substeps
Each case stores ``<case>_<field>_in`` / ``<case>_<field>_out`` for x, v, C, F, Jp,
``<case>_mat``, ``<case>_grid`` (the last substep's grid after P2G), and
``<case>_materials`` (rows: kind, volume, density, E, nu, hardening, lo, hi) plus
``<case>_params`` (dt, N, nsteps).
"""
import ctypes

import numpy as np

SNOW = 0


def _state(rng, n, N, deform):
    x = rng.uniform(0.25, 0.75, (n, 3)).astype(np.float32)
    v = (0.5 * rng.standard_normal((n, 3))).astype(np.float32)
    C = (0.5 * N * rng.standard_normal((n, 3, 3)) * 0.1).astype(np.float32)
    F = (np.eye(3)[None] + deform * rng.standard_normal((n, 3, 3))).astype(np.float32)
    Jp = rng.uniform(0.95, 1.05, n).astype(np.float32)
    return {"x": x, "v": v, "C": C, "F": F, "Jp": Jp}


def _run(lib, st, mat, materials, dt, N, nsteps):
    n = st["x"].shape[0]
    out = {k: np.ascontiguousarray(st[k].copy()) for k in st}
    grid = np.zeros((N, N, N, 4), np.float32)
    mrows = np.ascontiguousarray(np.array([m[1:] for m in materials], np.float32))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = lib.ref_substep(ctypes.c_int64(n), P(out["x"]), P(out["v"]), P(out["C"]), P(out["F"]), P(out["Jp"]),
                         P(np.ascontiguousarray(mat)), P(mrows), ctypes.c_int(len(materials)), ctypes.c_float(dt),
                         ctypes.c_int(N), ctypes.c_int(nsteps), P(grid))
    assert rc == 0
    return out, grid


def make(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.ref_substep.restype = ctypes.c_int
    elastic = lambda vol: (SNOW, vol, 1000.0, 1e4, 0.3, 0.0, 0.0, 1e30)  # noqa: E731
    snow = lambda vol: (SNOW, vol, 700.0, 1.4e5, 0.2, 10.0, 1.0 - 2.5e-2, 1.0 + 7.5e-3)  # noqa: E731
    cases = []
    rng = np.random.default_rng(2024)
    st = _state(rng, 2000, 16, 0.02)
    mat = np.zeros(2000, np.uint8)
    cases += [("elastic1", st, mat, [elastic(1.0 / 2000)], 1e-4, 16, 1),
              ("elastic4", st, mat, [elastic(1.0 / 2000)], 1e-4, 16, 4)]
    st = _state(rng, 2000, 16, 0.04)
    cases += [("snow1", st, mat, [snow(1.0 / 2000)], 1e-4, 16, 1),
              ("snow3", st, mat, [snow(1.0 / 2000)], 1e-4, 16, 3)]
    st = _state(rng, 3000, 24, 0.03)
    mat = (rng.uniform(size=3000) < 0.5).astype(np.uint8)
    cases += [("mixed2", st, mat, [snow(1.0 / 3000), elastic(1.0 / 3000)], 5e-5, 24, 2)]
    out = {}
    for name, st, mat, materials, dt, N, nsteps in cases:
        res, grid = _run(lib, st, mat, materials, dt, N, nsteps)
        for k in st:
            out[f"{name}_{k}_in"] = st[k]
            out[f"{name}_{k}_out"] = res[k]
        out[f"{name}_mat"] = mat
        out[f"{name}_grid"] = grid
        out[f"{name}_materials"] = np.array(materials, np.float64)
        out[f"{name}_params"] = np.array([dt, N, nsteps], np.float64)
    out["cases"] = np.array([c[0] for c in cases])
    return out
