"""Shared comparison helpers for the parity tests."""
import os

import numpy as np

FIELDS = ("x", "v", "C", "F", "Jp")


def rel_err(a, b, scale=0.0):
    """Norm-wise relative error ||a - b|| / max(||b||, scale * sqrt(size)).

    `scale` is the field's natural magnitude; it keeps fields that are zero up to
    rounding (C of a body at rest) from dividing noise by noise."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.linalg.norm(b), scale * np.sqrt(b.size), 1e-30)
    return float(np.linalg.norm(a - b) / den)


def field_scales(state, params):
    """Natural magnitude of each field: domain size for x, the largest speed (at
    least dt|g|) for v, 4 N |v| for C (|C| <= D dx |v|), 1 for F and Jp."""
    vmax = max(float(np.abs(state["v"]).max()), abs(params["dt"] * params.get("gravity", -9.81)))
    return {"x": 1.0, "v": vmax, "C": 4.0 * params["N"] * vmax, "F": 1.0, "Jp": 1.0}


def compare_states(a, b, params, ref_state=None):
    sc = field_scales(ref_state if ref_state is not None else b, params)
    return {k: rel_err(a[k], b[k], sc[k]) for k in FIELDS}


GOLDEN_SUBSTEP = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_substep.npz")


def golden_substep_cases():
    """The reference-policy substep vectors (tests/golden/ref_substep.npz) as
    (name, cfg, nsteps, expected_state, expected_grid_after_p2g); cfg is in the form
    ``Simulation.from_config`` and the oracle take."""
    from mpm_gb300.materials import Material

    d = np.load(GOLDEN_SUBSTEP)
    cases = []
    for name in (str(c) for c in d["cases"]):
        dt, N, nsteps = d[name + "_params"]
        state = {k: d[f"{name}_{k}_in"] for k in FIELDS}
        state["mat"] = d[name + "_mat"]
        expect = {k: d[f"{name}_{k}_out"] for k in FIELDS}
        mats = [Material(int(r[0]), *(float(q) for q in r[1:])) for r in d[name + "_materials"]]
        cfg = {"params": {"dt": float(dt), "N": int(N), "g2p_guard": 1}, "materials": mats, "state": state}
        cases.append((name, cfg, int(nsteps), expect, d[name + "_grid"]))
    return cases


def icosphere(subdivisions=2):
    """A closed triangle mesh of the unit sphere: an icosahedron with each triangle split
    into four `subdivisions` times, vertices pushed onto the sphere; outward winding."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]]
    V = [list(np.asarray(v, np.float64) / np.linalg.norm(v)) for v in V]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = (np.asarray(V[a]) + np.asarray(V[b])) / 2.0
                V.append(list(m / np.linalg.norm(m)))
                mid[key] = len(V) - 1
            return mid[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        F = nf
    return np.asarray(V, np.float32), np.asarray(F, np.int32)


def write_obj(path, V, F, quads=False):
    with open(path, "w") as f:
        f.write("# test mesh\n")
        for v in V:
            f.write(f"v {v[0]:.7f} {v[1]:.7f} {v[2]:.7f}\n")
        for tri in F:
            f.write("f " + " ".join(f"{i + 1}/{i + 1}" for i in tri) + "\n")


def open_icosphere(subdivisions=3, cut=0.6):
    """The icosphere with the triangles of its cap y > cut removed: a mesh with a hole."""
    V, F = icosphere(subdivisions)
    keep = V[F].max(axis=1)[:, 1] <= cut
    return V, F[keep]


def two_spheres(subdivisions=2):
    """Two overlapping closed icospheres in one mesh (centres 0.6 apart, radius 1): ray parity
    calls their overlap outside (two crossings), the winding number 2."""
    V, F = icosphere(subdivisions)
    V2 = V + np.array([0.6, 0.0, 0.0], np.float32)
    return np.concatenate([V, V2]).astype(np.float32), np.concatenate([F, F + V.shape[0]]).astype(np.int32)
