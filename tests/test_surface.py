"""CPU tests of the surface-reconstruction oracle (oracle/surface_oracle.cpp): the
distance field of fillVoxelGrid_distance (include/mesh_builder.h:89-137) bit for bit
against the reference's own header compiled for the host (tests/golden/ref_mesh.npz) and
against a numpy float32 restatement, and the marching-tetrahedra surface checked for the
properties of a closed, outward-oriented surface."""
import numpy as np
import pytest

from surface_checks import (ambiguous_mask, cube_loop_mismatches, cube_masks, edge_balance, enclosed_volume,
                            golden_mesh_cases, golden_meshes, matches_golden, vertices_match, weld)

MESH_CASES = golden_mesh_cases()
MESHES = golden_meshes()


@pytest.mark.parametrize("case", MESHES, ids=[c[0] for c in MESHES])
def test_mesh_vertices_match_reference_golden(oracle_lib, case):
    """The vertex list of MeshBuilder::computeMesh (libigl's marching cubes on
    S = radius voxel_dx - field, scaled by voxel_dx; include/mesh_builder.h:165-211), bit for
    bit and in the same order, and the same face count."""
    name, x, N, G, r, V, F, sha, nv, nf = case
    vdx = oracle_lib.voxel_dx(N, float(np.float32(1.0 / N)), G)
    Vo, Fo = oracle_lib.surface_indexed(oracle_lib.distance_field(x, G, r, vdx), r, vdx)
    assert vertices_match(Vo, V, sha, nv)
    assert len(Fo) == nf


@pytest.mark.parametrize("case", [c for c in MESHES if c[6] is not None], ids=[c[0] for c in MESHES if c[6] is not None])
def test_mesh_faces_bound_the_reference_loops(oracle_lib, case):
    """Per cube, the oracle's faces and libigl's bound the same directed loops of edge
    vertices (same segments on every cube face, same orientation), ambiguous faces
    included; only the triangulation inside a loop may differ."""
    name, x, N, G, r, V, F, sha, nv, nf = case
    vdx = oracle_lib.voxel_dx(N, float(np.float32(1.0 / N)), G)
    field = oracle_lib.distance_field(x, G, r, vdx)
    _, Fo = oracle_lib.surface_indexed(field, r, vdx)
    counts, _ = oracle_lib.surface_table()
    masks = cube_masks(field, r, vdx)
    bad, cubes = cube_loop_mismatches(Fo, F, masks, counts)
    assert cubes > 0 and bad == 0
    if name.startswith("cloud"):
        assert sum(ambiguous_mask(int(m)) for m in masks if counts[m]) > 10


def test_loop_check_detects_a_reversed_face(oracle_lib):
    name, x, N, G, r, V, F, sha, nv, nf = next(c for c in MESHES if c[6] is not None)
    vdx = oracle_lib.voxel_dx(N, float(np.float32(1.0 / N)), G)
    field = oracle_lib.distance_field(x, G, r, vdx)
    _, Fo = oracle_lib.surface_indexed(field, r, vdx)
    counts, _ = oracle_lib.surface_table()
    Fo = Fo.copy()
    Fo[len(Fo) // 2] = Fo[len(Fo) // 2][::-1]
    bad, _ = cube_loop_mismatches(Fo, F, cube_masks(field, r, vdx), counts)
    assert bad == 1


def test_oracle_table_is_closed_and_oriented(oracle_lib):
    """Each mask's triangles close around the crossed edges: every crossed edge slot is
    used, and the triangles' boundary is a set of loops."""
    counts, slots = oracle_lib.surface_table()
    edges = ((0, 1), (1, 2), (3, 2), (0, 3), (4, 5), (5, 6), (7, 6), (4, 7), (0, 4), (1, 5), (2, 6), (3, 7))
    for m in range(256):
        crossed = {e for e, (a, b) in enumerate(edges) if ((m >> a) ^ (m >> b)) & 1}
        T = slots[m][: 3 * counts[m]].reshape(-1, 3)
        assert set(T.ravel().tolist()) == crossed
        assert counts[m] <= 5


@pytest.mark.parametrize("case", MESH_CASES, ids=[c[0] for c in MESH_CASES])
def test_distance_field_matches_reference_golden(oracle_lib, case):
    """The reference's fillVoxelGrid_distance, called as MeshBuilder::computeMesh calls it
    (include/mesh_builder.h:167-174), on seeded particles reaching past both faces of the
    grid; the largest case is the reference's default mesh grid (G = 250, radius 5)."""
    name, x, N, G, r, vdx, field, sha = case
    assert oracle_lib.voxel_dx(N, float(np.float32(1.0 / N)), G) == vdx
    assert matches_golden(oracle_lib.distance_field(x, G, r, vdx), field, sha)


@pytest.mark.parametrize("stored", [True, False])
def test_golden_distance_check_detects_a_changed_node(oracle_lib, stored):
    name, x, N, G, r, vdx, field, sha = next(c for c in MESH_CASES if (c[6] is not None) == stored)
    f = oracle_lib.distance_field(x, G, r, vdx)
    hit = np.argwhere(f < f.max())[0]
    f[tuple(hit)] = np.nextafter(f[tuple(hit)], np.float32(0))
    assert not matches_golden(f, field, sha)


def numpy_distance_field(x, G, radius, vdx):
    """fillVoxelGrid_distance in numpy float32 (every operation rounded to float)."""
    f32 = np.float32
    dx = f32(vdx)
    cutoff = f32((radius + 1) * vdx)
    field = np.full((G, G, G), cutoff, np.float32)
    r = f32(cutoff / dx)
    for p in np.asarray(x, np.float32):
        g = p / dx
        lo = np.maximum(0, (g - r).astype(np.int32))
        hi = np.minimum(G, (g + f32(r + f32(1))).astype(np.int32))
        if np.any(hi <= lo):
            continue
        nodes = [np.arange(lo[c], hi[c]).astype(np.float32) * dx for c in range(3)]
        d = [(p[c] - nodes[c]).astype(np.float32) for c in range(3)]
        s = d[0][:, None, None] ** 2 + (d[1][None, :, None] ** 2 + d[2][None, None, :] ** 2)
        dist = np.sqrt(s.astype(np.float32))
        box = field[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        np.minimum(box, dist, out=box)
    return field


def ball(n, center, radius, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = radius * rng.random(n) ** (1.0 / 3.0)
    return (np.asarray(center) + u * r[:, None]).astype(np.float32)


@pytest.mark.parametrize("G,radius", [(24, 2), (33, 3), (16, 0)])
def test_distance_field_matches_numpy_restatement(oracle_lib, G, radius):
    rng = np.random.default_rng(G)
    x = rng.random((400, 3)).astype(np.float32)
    x[:5] = [[0, 0, 0], [1, 1, 1], [0.999, 0.0, 0.5], [1e-7, 0.5, 0.999999], [0.5, 0.5, 0.5]]
    vdx = oracle_lib.voxel_dx(32, 1.0 / 32, G)
    a = oracle_lib.distance_field(x, G, radius, vdx)
    b = numpy_distance_field(x, G, radius, vdx)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


def test_voxel_dx_follows_reference_types(oracle_lib):
    # params.N * params.dx is a float product, then divided in double by the grid side
    dx = float(np.float32(1.0 / 60))
    assert oracle_lib.voxel_dx(60, dx, 250) == float(np.float32(60) * np.float32(dx)) / 250.0


def test_empty_field_has_no_surface(oracle_lib):
    f = oracle_lib.distance_field(np.zeros((0, 3), np.float32), 12, 2, 1 / 12)
    assert np.all(f == np.float32(3 / 12))
    assert oracle_lib.surface_mesh(f, 2, 1 / 12).shape == (0, 3, 3)


def test_single_particle_gives_closed_outward_surface(oracle_lib):
    G, radius = 20, 3
    vdx = 1.0 / G
    f = oracle_lib.distance_field(np.array([[0.51, 0.49, 0.503]], np.float32), G, radius, vdx)
    tris = oracle_lib.surface_mesh(f, radius, vdx)
    assert len(tris) > 50
    V, F = weld(tris)
    assert edge_balance(F) == 0
    vol = enclosed_volume(tris)
    r = radius * vdx
    assert 0.8 * (4 / 3) * np.pi * r ** 3 < vol < 1.05 * (4 / 3) * np.pi * r ** 3
    # every vertex lies on the level set up to the linear interpolation's error
    d = np.linalg.norm(V - np.array([0.51, 0.49, 0.503]), axis=1)
    assert np.all(np.abs(d - r) < 0.5 * vdx)


def test_ball_of_particles_is_closed_with_the_expected_volume(oracle_lib):
    G, radius = 48, 2
    vdx = 1.0 / G
    x = ball(20000, (0.5, 0.5, 0.5), 0.25, 1)
    f = oracle_lib.distance_field(x, G, radius, vdx)
    tris = oracle_lib.surface_mesh(f, radius, vdx)
    V, F = weld(tris)
    assert edge_balance(F) == 0
    # the surface sits about radius voxels outside the particles
    R = 0.25 + radius * vdx
    assert abs(enclosed_volume(tris) / ((4 / 3) * np.pi * R ** 3) - 1.0) < 0.06


def test_surface_touching_the_grid_edge_stays_open_there(oracle_lib):
    # a particle cluster at the domain corner: the level set is cut by the grid boundary
    G, radius = 16, 2
    vdx = 1.0 / G
    f = oracle_lib.distance_field(np.array([[0.01, 0.01, 0.01]], np.float32), G, radius, vdx)
    tris = oracle_lib.surface_mesh(f, radius, vdx)
    assert len(tris) > 0
    assert enclosed_volume(tris) != 0.0


def test_mesh_builder_writes_welded_obj(tmp_path, oracle_lib):
    from mpm_gb300.mesh_builder import weld as w, write_obj

    G, radius = 16, 2
    f = oracle_lib.distance_field(np.array([[0.5, 0.5, 0.5]], np.float32), G, radius, 1 / G)
    tris = oracle_lib.surface_mesh(f, radius, 1 / G)
    V, F = w(tris)
    p = tmp_path / "m.obj"
    write_obj(str(p), V, F)
    lines = p.read_text().splitlines()
    assert sum(l.startswith("v ") for l in lines) == len(V)
    assert sum(l.startswith("f ") for l in lines) == len(F)
    assert F.min() == 0 and F.max() == len(V) - 1
    # welded vertices: Euler characteristic of a sphere
    E = len(np.unique(np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1), axis=0))
    assert len(V) - E + len(F) == 2
