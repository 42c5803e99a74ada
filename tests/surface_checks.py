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
    for key in sorted(k for k in d.files if k.endswith("_params") and not k.startswith("mesh_")):
        name = key[: -len("_params")]
        N, G, r = (int(v) for v in d[key])
        field = d[name + "_field"] if name + "_field" in d.files else None
        sha = str(d[name + "_sha256"]) if name + "_sha256" in d.files else None
        out.append((name, d[name + "_x"], N, G, r, float(d[name + "_voxel_dx"]), field, sha))
    return out


def golden_meshes():
    """[(name, x, N, G, radius, V or None, F or None, V sha256 or None, nv, nf)]: the
    meshes MeshBuilder::computeMesh writes for seeded particle sets (ref_mesh.npz)."""
    d = np.load(GOLDEN_MESH)
    out = []
    for key in sorted(k for k in d.files if k.startswith("mesh_") and k.endswith("_params")):
        name = key[: -len("_params")]
        N, G, r = (int(v) for v in d[key])
        V = d[name + "_V"] if name + "_V" in d.files else None
        F = d[name + "_F"] if name + "_F" in d.files else None
        sha = str(d[name + "_Vsha256"]) if name + "_Vsha256" in d.files else None
        nv = len(V) if V is not None else int(d[name + "_nv"])
        out.append((name[len("mesh_"):], d[name + "_x"], N, G, r, V, F, sha, nv, int(d[name + "_nf"])))
    return out


def vertices_match(V, golden_V, sha, nv):
    """Bit-for-bit equality of a vertex list with the stored one (or its sha256)."""
    V = np.ascontiguousarray(V, np.float64)
    if golden_V is not None:
        return V.shape == golden_V.shape and np.array_equal(V.view(np.uint64), golden_V.view(np.uint64))
    return len(V) == nv and hashlib.sha256(V.tobytes()).hexdigest() == sha


# libigl's cube corners (di, dj, dk) and the cube faces' corner cycles
MC_CORNERS = ((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0), (1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0))
MC_FACES = ((0, 1, 2, 3), (4, 7, 6, 5), (0, 4, 5, 1), (3, 2, 6, 7), (0, 3, 7, 4), (1, 5, 6, 2))


def cube_masks(field, radius, vdx):
    """Inside-corner mask per cube ((G-1)^3, cube order): bit n when S = radius vdx -
    field > 0 at libigl's corner n."""
    G = field.shape[0]
    inside = (radius * vdx - field.astype(np.float64)) > 0
    m = np.zeros((G - 1,) * 3, np.int32)
    for n, (a, b, c) in enumerate(MC_CORNERS):
        m |= inside[a:a + G - 1, b:b + G - 1, c:c + G - 1].astype(np.int32) << n
    return m.ravel()


def ambiguous_mask(m):
    """Whether the cube with inside-corner mask m has a face with two opposite inside corners."""
    for q in MC_FACES:
        b = [(m >> c) & 1 for c in q]
        if b[0] == b[2] and b[1] == b[3] and b[0] != b[1]:
            return True
    return False


def cube_loop_mismatches(F_a, F_b, masks, counts):
    """Cubes whose faces in F_a and F_b (both in cube order, counts[mask] faces per cube)
    bound different directed edge loops; returns (mismatching cubes, surface cubes)."""
    per = counts[masks]
    off = np.concatenate([[0], np.cumsum(per)])
    if off[-1] != len(F_a) or off[-1] != len(F_b):
        return -1, int(np.count_nonzero(per))

    def boundary(T):
        e = set()
        for t in T:
            for x, y in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
                x, y = int(x), int(y)
                if (y, x) in e:
                    e.remove((y, x))
                else:
                    e.add((x, y))
        return e

    bad = 0
    nz = np.nonzero(per)[0]
    for c in nz:
        bad += boundary(F_a[off[c]:off[c + 1]]) != boundary(F_b[off[c]:off[c + 1]])
    return bad, len(nz)


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
