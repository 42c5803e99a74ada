"""Shared comparison helpers for the parity tests."""
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
