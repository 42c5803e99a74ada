"""Test infrastructure: a CPU restatement of the reference's Laplacian mesh smoothing.

MeshBuilder::smoothMesh (include/mesh_builder.h:212-245) makes one implicit smoothing step
with libigl (vendored under include/igl/) and rescales the result to unit area:

    L = cotmatrix(V, F)                                  cotmatrix.cpp:39-78
    M = massmatrix(V, F, MASSMATRIX_TYPE_BARYCENTRIC)    massmatrix.cpp:47-48,
                                                         massmatrix_intrinsic.cpp:48-64
    U = SimplicialLLT(M - 0.001 L).solve(M V)
    U /= sqrt(0.5 * doublearea(U, F).sum())              doublearea.cpp:33-57

(the gradient operator G, K and the barycenters BC it also forms are unused).  The entries
are restated here with numpy in double, in libigl's expressions:

* squared_edge_lengths.cpp:39-41: l2[:, 0] = |V1 - V2|^2, l2[:, 1] = |V2 - V0|^2,
  l2[:, 2] = |V0 - V1|^2 (edge e opposite corner e);
* doublearea.cpp:147-197 (from edge lengths, the one cotmatrix_entries and
  massmatrix_intrinsic use): Kahan's form of Heron's formula on the lengths sorted in
  decreasing order, dblA = 2 * 0.25 * sqrt(arg), NaN replaced by 0;
* cotmatrix_entries.cpp:39-58: C[:, e] = (l2_a + l2_b - l2_e) / dblA / 4;
* cotmatrix.cpp:39-78: for edges (1,2), (2,0), (0,1) of each face, L(s, d) and L(d, s) get
  +C, L(s, s) and L(d, d) get -C;
* massmatrix_intrinsic.cpp:56-64: M(v, v) += dblA / 6 for each corner v.

The linear system is solved by a direct sparse LU (scipy's spsolve) in place of Eigen's
sparse Cholesky; both solve the same symmetric positive definite system to rounding.

Parity pin: the reference's smoothing cannot be compiled here (it needs Eigen's sparse
module and libigl's compiled sparse helpers, neither of which is vendored), so these
functions are pinned by the identities libigl's definitions imply, checked in the tests:
C[:, e] = cot(angle e) / 2, L annihilates constants and reproduces linear functions at the
interior vertices of a planar mesh, the mass matrix sums to the surface area, and the
rescaled result has unit area.  Only the tests and the CPU baseline use this module.
"""
from __future__ import annotations

import numpy as np

EDGES = ((1, 2), (2, 0), (0, 1))  # cotmatrix.cpp:39-42


def squared_edge_lengths(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """(m, 3) squared lengths, column e = the edge opposite corner e."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    P = [V[F[:, k]] for k in range(3)]
    return np.stack([((P[a] - P[b]) ** 2).sum(axis=1) for a, b in EDGES], axis=1)


def doublearea_from_lengths(l: np.ndarray, nan_replacement: float = 0.0) -> np.ndarray:
    """Twice the triangle areas from edge lengths by Kahan's Heron (doublearea.cpp:160-196)."""
    s = -np.sort(-np.asarray(l, np.float64), axis=1)  # decreasing
    l0, l1, l2 = s[:, 0], s[:, 1], s[:, 2]
    with np.errstate(invalid="ignore"):
        arg = (l0 + (l1 + l2)) * (l2 - (l0 - l1)) * (l2 + (l0 - l1)) * (l0 + (l1 - l2))
        dblA = 2.0 * 0.25 * np.sqrt(arg)
    dblA[np.isnan(dblA)] = nan_replacement
    return dblA


def doublearea(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Twice the triangle areas of a 3-D mesh from the projected areas (doublearea.cpp:33-57)."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    A, B, C = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    acc = np.zeros(len(F))
    for d in range(3):
        x, y = d, (d + 1) % 3
        rx, sx = A[:, x] - C[:, x], B[:, x] - C[:, x]
        ry, sy = A[:, y] - C[:, y], B[:, y] - C[:, y]
        acc += (rx * sy - ry * sx) ** 2
    return np.sqrt(acc)


def cotmatrix_entries(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """(m, 3) half cotangents of the angles opposite each edge (cotmatrix_entries.cpp:39-58)."""
    l2 = squared_edge_lengths(V, F)
    dblA = doublearea_from_lengths(np.sqrt(l2))
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.stack([(l2[:, 1] + l2[:, 2] - l2[:, 0]) / dblA / 4.0,
                         (l2[:, 2] + l2[:, 0] - l2[:, 1]) / dblA / 4.0,
                         (l2[:, 0] + l2[:, 1] - l2[:, 2]) / dblA / 4.0], axis=1)


def cotmatrix(V: np.ndarray, F: np.ndarray):
    """The cotangent Laplacian L (n x n, scipy CSR; cotmatrix.cpp:62-78)."""
    import scipy.sparse as sp

    F = np.asarray(F, np.int64)
    n = len(V)
    C = cotmatrix_entries(V, F)
    rows, cols, vals = [], [], []
    for e, (a, b) in enumerate(EDGES):
        s, d, c = F[:, a], F[:, b], C[:, e]
        rows += [s, d, s, d]
        cols += [d, s, s, d]
        vals += [c, c, -c, -c]
    return sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n)).tocsr()


def massmatrix_barycentric(V: np.ndarray, F: np.ndarray):
    """The lumped barycentric mass matrix (diagonal, scipy CSR; massmatrix_intrinsic.cpp:48-64)."""
    import scipy.sparse as sp

    F = np.asarray(F, np.int64)
    dblA = doublearea_from_lengths(np.sqrt(squared_edge_lengths(V, F)))
    m = np.zeros(len(V))
    for k in range(3):
        np.add.at(m, F[:, k], dblA / 6.0)
    return sp.diags(m).tocsr()


def smooth_mesh(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """MeshBuilder::smoothMesh (include/mesh_builder.h:212-245): the smoothed, unit-area
    vertices.  A vertex that no face uses has a zero row in M - 0.001 L (the reference's
    Cholesky factorisation fails on it); here it keeps its position, rescaled like the rest."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    V = np.asarray(V, np.float64)
    L = cotmatrix(V, F)
    M = massmatrix_barycentric(V, F)
    unused = (M.diagonal() == 0.0).astype(np.float64)
    S = (M - 0.001 * L + sp.diags(unused)).tocsc()
    B = M @ V + unused[:, None] * V
    U = np.asarray(spla.spsolve(S, B))  # one factorisation for the three coordinates
    area = 0.5 * doublearea(U, F).sum()
    return U / np.sqrt(area)
