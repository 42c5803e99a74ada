"""CPU tests of the Laplacian smoothing oracle (oracle/smooth_oracle.py), the restatement of
MeshBuilder::smoothMesh (include/mesh_builder.h:212-245) and the libigl operators it calls.

The reference's smoothing cannot be built here (Eigen's sparse module is not vendored), so
the oracle is pinned by identities that libigl's definitions imply: the cotangent entries
are half the cotangents of the opposite angles, the Laplacian annihilates constants and
reproduces linear functions at the interior vertices of a planar mesh, the lumped masses
sum to the surface area, Heron's area equals the projected one, and the result has unit
area."""
import numpy as np
import pytest

from helpers import icosphere, open_icosphere

pytest.importorskip("scipy")
from oracle import smooth_oracle as so  # noqa: E402


def _planar_mesh(n=7, seed=0):
    """A jittered n x n grid triangulated in the plane z = 0, then rotated and shifted;
    returns V, F and the mask of interior vertices."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    P = np.stack([i.ravel(), j.ravel(), np.zeros(n * n)], axis=1).astype(np.float64)
    interior = ((i > 0) & (i < n - 1) & (j > 0) & (j < n - 1)).ravel()
    P[interior, :2] += rng.uniform(-0.25, 0.25, size=(interior.sum(), 2))
    F = []
    for a in range(n - 1):
        for b in range(n - 1):
            v00, v01, v10, v11 = a * n + b, a * n + b + 1, (a + 1) * n + b, (a + 1) * n + b + 1
            F += [[v00, v10, v11], [v00, v11, v01]]
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    V = P @ q.T + rng.normal(size=3)
    return V, np.asarray(F, np.int32), interior


def _compact(V, F):
    """The mesh without the vertices no face uses."""
    used, F2 = np.unique(F, return_inverse=True)
    return np.asarray(V, np.float64)[used], F2.reshape(-1, 3).astype(np.int32)


def test_cot_entries_are_half_cotangents():
    rng = np.random.default_rng(1)
    V = rng.normal(size=(300, 3))
    F = np.arange(300, dtype=np.int32).reshape(-1, 3)
    C = so.cotmatrix_entries(V, F)
    for e, (a, b) in enumerate(so.EDGES):
        apex = 3 - a - b  # the corner opposite edge (a, b)
        u = V[F[:, a]] - V[F[:, apex]]
        w = V[F[:, b]] - V[F[:, apex]]
        cot = (u * w).sum(axis=1) / np.linalg.norm(np.cross(u, w), axis=1)
        np.testing.assert_allclose(C[:, e], 0.5 * cot, rtol=1e-9, atol=1e-12)


def test_heron_area_equals_projected_area():
    rng = np.random.default_rng(2)
    V = rng.normal(size=(600, 3))
    F = np.arange(600, dtype=np.int32).reshape(-1, 3)
    heron = so.doublearea_from_lengths(np.sqrt(so.squared_edge_lengths(V, F)))
    np.testing.assert_allclose(heron, so.doublearea(V, F), rtol=1e-10)


def test_degenerate_face_area_is_zero_and_entries_not_finite():
    V = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float64)  # collinear
    F = np.array([[0, 1, 2]], np.int32)
    assert so.doublearea_from_lengths(np.sqrt(so.squared_edge_lengths(V, F)))[0] == 0.0
    assert not np.all(np.isfinite(so.cotmatrix_entries(V, F)))


def test_laplacian_constants_and_linear_precision():
    V, F, interior = _planar_mesh()
    L = so.cotmatrix(V, F)
    assert abs(L - L.T).max() == 0.0
    np.testing.assert_allclose(L @ np.ones(len(V)), 0.0, atol=1e-12)
    rng = np.random.default_rng(3)
    for _ in range(3):
        f = V @ rng.normal(size=3) + rng.normal()
        np.testing.assert_allclose((L @ f)[interior], 0.0, atol=1e-11)
        assert np.abs((L @ f)[~interior]).max() > 1e-6  # the boundary rows do not vanish


def test_laplacian_is_negative_semidefinite():
    V, F = icosphere(2)
    L = so.cotmatrix(V.astype(np.float64), F).toarray()
    w = np.linalg.eigvalsh(L)
    assert w.max() < 1e-10 * np.abs(w).max()


def test_mass_sums_to_area():
    for V, F in (icosphere(2), open_icosphere(2)):
        M = so.massmatrix_barycentric(V, F)
        np.testing.assert_allclose(M.diagonal().sum(), 0.5 * so.doublearea(V, F).sum(), rtol=1e-12)


def test_smooth_mesh_unit_area_and_sphere_stays_round():
    V, F = icosphere(3)
    U = so.smooth_mesh(V, F)
    np.testing.assert_allclose(0.5 * so.doublearea(U, F).sum(), 1.0, rtol=1e-12)
    r = np.linalg.norm(U - U.mean(axis=0), axis=1)
    assert r.std() < 1e-2 * r.mean()  # smoothing a round sphere moves its vertices radially
    # the smoothed sphere's area is 1: its radius is close to sqrt(1 / (4 pi))
    assert abs(r.mean() - (1.0 / (4.0 * np.pi)) ** 0.5) < 0.01


def test_smooth_mesh_solves_the_reference_system():
    V, F = _compact(*open_icosphere(3))
    V = V * 3.0
    U = so.smooth_mesh(V, F)
    # a dense solve of (M - 0.001 L) X = M V, rescaled to unit area
    L = so.cotmatrix(V, F).toarray()
    M = so.massmatrix_barycentric(V, F).toarray()
    X = np.linalg.solve(M - 0.001 * L, M @ V)
    np.testing.assert_allclose(U, X / np.sqrt(0.5 * so.doublearea(X, F).sum()), rtol=1e-9, atol=1e-12)


def test_smooth_mesh_unused_vertex_keeps_position():
    V, F = icosphere(2)
    V = np.vstack([V.astype(np.float64), [[5.0, 6.0, 7.0]]])
    U = so.smooth_mesh(V, F)
    U0 = so.smooth_mesh(V[:-1], F)
    np.testing.assert_allclose(U[:-1], U0, rtol=1e-12, atol=1e-14)
    # the isolated vertex is divided by the same sqrt(area) as the rest
    L = so.cotmatrix(V[:-1], F).toarray()
    M = so.massmatrix_barycentric(V[:-1], F).toarray()
    X = np.linalg.solve(M - 0.001 * L, M @ V[:-1])
    np.testing.assert_allclose(U[-1], V[-1] / np.sqrt(0.5 * so.doublearea(X, F).sum()), rtol=1e-10)
