"""Size-independent checks of a triangle soup (T, 3, 3): closed, consistently
oriented, outward, and its enclosed volume."""
import numpy as np


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
