"""Size-independent checks of a triangle soup (T, 3, 3): closed, consistently
oriented, outward, and its enclosed volume; and the golden distance fields of the
reference's own include/mesh_builder.h (tests/golden/ref_mesh.npz)."""
import hashlib
import os

import numpy as np

GOLDEN_MESH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_mesh.npz")


def golden_mesh_cases():
    """[(name, x, N, G, radius, voxel_dx, field or None, sha256 or None)] from ref_mesh.npz."""
    d = np.load(GOLDEN_MESH)
    out = []
    for key in sorted(k for k in d.files if k.endswith("_params")):
        name = key[: -len("_params")]
        N, G, r = (int(v) for v in d[key])
        field = d[name + "_field"] if name + "_field" in d.files else None
        sha = str(d[name + "_sha256"]) if name + "_sha256" in d.files else None
        out.append((name, d[name + "_x"], N, G, r, float(d[name + "_voxel_dx"]), field, sha))
    return out


def matches_golden(field, golden_field, sha):
    """Bit-for-bit equality with the stored field, or with the stored field's sha256."""
    f = np.ascontiguousarray(field, np.float32)
    if golden_field is not None:
        return np.array_equal(f.view(np.uint32), np.asarray(golden_field, np.float32).view(np.uint32))
    return hashlib.sha256(f.tobytes()).hexdigest() == sha


def weld(tris):
    from mpm_gb300.mesh_builder import weld as _weld

    return _weld(tris)


def edge_balance(F):
    """Directed edges that are not matched by their reverse (0 for a closed, consistently
    oriented surface)."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    e = e[e[:, 0] != e[:, 1]]
    fwd = e[:, 0].astype(np.int64) * (1 << 32) + e[:, 1]
    rev = e[:, 1].astype(np.int64) * (1 << 32) + e[:, 0]
    uf, cf = np.unique(fwd, return_counts=True)
    ur, cr = np.unique(rev, return_counts=True)
    a = dict(zip(uf.tolist(), cf.tolist()))
    b = dict(zip(ur.tolist(), cr.tolist()))
    keys = set(a) | set(b)
    return sum(abs(a.get(k, 0) - b.get(k, 0)) for k in keys)


def enclosed_volume(tris):
    """Signed volume by the divergence theorem (positive for outward normals)."""
    t = tris.astype(np.float64)
    return float(np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])).sum() / 6.0)
