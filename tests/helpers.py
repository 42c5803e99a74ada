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
