"""GPU tests of surface reconstruction (mpm_surface_distance / mpm_surface_mesh /
mpm_surface_mesh_indexed): the distance field of fillVoxelGrid_distance
(include/mesh_builder.h:89-137) bit for bit against the oracle and the reference's own
header; the marching-cubes vertices bit for bit and the faces index for index against the
oracle, the vertices also against the reference's MeshBuilder::computeMesh with libigl's
marching cubes; and a simulated body's surface closed and outward."""
import numpy as np
import pytest

from surface_checks import (cube_loop_mismatches, cube_masks, edge_balance, enclosed_volume, golden_mesh_cases,
                            golden_meshes, matches_golden, vertices_match, weld)

MESH_CASES = golden_mesh_cases()
MESHES = golden_meshes()

pytestmark = pytest.mark.gpu


def _sim(x, N=32, liquid=False):
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    sim = Simulation(dt=1e-4, N=N, sort_interval=4)
    vol = 1.0 / max(len(x), 1)
    sim.set_materials([M.liquid(vol) if liquid else M.elastic(vol)])
    sim.upload({"x": x})
    return sim


def _ball(n, center, radius, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = radius * rng.random(n) ** (1.0 / 3.0)
    return (np.asarray(center) + u * r[:, None]).astype(np.float32)


@pytest.mark.parametrize("N,G,radius", [(32, 40, 2), (60, 64, 5), (24, 17, 0), (32, 2, 1)])
def test_distance_field_matches_oracle(gpu_lib, oracle_lib, N, G, radius):
    rng = np.random.default_rng(G + radius)
    x = rng.random((3000, 3)).astype(np.float32)
    x[:4] = [[0, 0, 0], [0.9999999, 0.9999999, 0.9999999], [0.5, 0.5, 0.5], [1e-7, 0.25, 0.75]]
    sim = _sim(x, N)
    g = sim.surface_distance(G, radius)
    dx = float(np.float32(1.0 / N))
    r = oracle_lib.distance_field(sim.download(("x",))["x"], G, radius, oracle_lib.voxel_dx(N, dx, G))
    assert np.array_equal(g.view(np.int32), r.view(np.int32))


@pytest.mark.parametrize("case", MESH_CASES, ids=[c[0] for c in MESH_CASES])
def test_distance_field_matches_reference_golden(gpu_lib, case):
    """The device field bit for bit against the reference's own fillVoxelGrid_distance
    (tests/golden/ref_mesh.npz), particles reaching past both faces of the grid."""
    name, x, N, G, r, vdx, field, sha = case
    sim = _sim(x, N)
    assert matches_golden(sim.surface_distance(G, r), field, sha)


@pytest.mark.parametrize("order,radius", [("sorted", 4), ("mixed", 4), ("sorted", 6), ("sorted", 7)])
def test_distance_field_of_cell_sorted_particles_matches_oracle(gpu_lib, oracle_lib, order, radius):
    # cell-sorted particles take the shared-tile path (two particles per warp up to radius
    # 6, one otherwise); a shuffled tail takes the direct one
    N, G = 40, 120
    x = _ball(60000, (0.5, 0.5, 0.5), 0.3, 5)
    sim = _sim(x, N)
    sim.sort()
    if order == "mixed":
        st = sim.download()
        perm = np.arange(len(x))
        tail = perm[len(x) // 2:]
        perm[len(x) // 2:] = np.random.default_rng(0).permutation(tail)
        sim.upload({k: v[perm] for k, v in st.items()})
    g = sim.surface_distance(G, radius)
    dx = float(np.float32(1.0 / N))
    r = oracle_lib.distance_field(sim.download(("x",))["x"], G, radius, oracle_lib.voxel_dx(N, dx, G))
    assert np.array_equal(g.view(np.int32), r.view(np.int32))


@pytest.mark.parametrize("G,radius", [(48, 2), (33, 3)])
def test_surface_triangles_match_oracle(gpu_lib, oracle_lib, G, radius):
    N = 32
    x = np.concatenate([_ball(30000, (0.5, 0.45, 0.5), 0.22, 1), _ball(3000, (0.2, 0.8, 0.3), 0.08, 2)])
    sim = _sim(x, N)
    tris = sim.surface_mesh(G, radius)
    field = sim.surface_distance(G, radius)
    dx = float(np.float32(1.0 / N))
    ref = oracle_lib.surface_mesh(field, radius, oracle_lib.voxel_dx(N, dx, G))
    assert len(tris) > 1000
    assert tris.shape == ref.shape
    assert np.array_equal(tris.view(np.int32), ref.view(np.int32))


@pytest.mark.parametrize("G,radius", [(48, 2), (33, 3), (300, 4), (512, 1), (2, 1)])
def test_indexed_mesh_matches_oracle(gpu_lib, oracle_lib, G, radius):
    """Vertices bit for bit and in order, faces index for index; G = 300 and 512 put two
    blocks of cubes on each row, so vertices are looked up across blocks, and 512 is the
    largest grid (cube coordinates up to 510 in the packed 10-bit fields)."""
    N = 32
    x = np.concatenate([_ball(30000, (0.5, 0.45, 0.5), 0.22, 1), _ball(3000, (0.2, 0.8, 0.3), 0.08, 2),
                        np.random.default_rng(G).random((300, 3)).astype(np.float32)])
    sim = _sim(x, N)
    V, F = sim.surface_indexed(G, radius)
    field = sim.surface_distance(G, radius)
    dx = float(np.float32(1.0 / N))
    Vo, Fo = oracle_lib.surface_indexed(field, radius, oracle_lib.voxel_dx(N, dx, G))
    assert V.shape == Vo.shape and np.array_equal(V.view(np.uint64), Vo.view(np.uint64))
    assert F.shape == Fo.shape and np.array_equal(F, Fo)
    if G > 2:
        assert len(F) > 1000 and F.min() == 0 and F.max() == len(V) - 1
    # the soup is the indexed mesh's faces with float vertices
    tris = sim.surface_mesh(G, radius)
    assert np.array_equal(tris.view(np.int32), V[F].astype(np.float32).view(np.int32))


@pytest.mark.parametrize("case", MESHES, ids=[c[0] for c in MESHES])
def test_indexed_mesh_matches_reference_golden(gpu_lib, oracle_lib, case):
    """The mesh of MeshBuilder::computeMesh with libigl's marching cubes
    (tests/golden/ref_mesh.npz): vertices bit for bit and in order, the face count, and per
    cube the same directed edge loops."""
    name, x, N, G, r, Vg, Fg, sha, nv, nf = case
    sim = _sim(x, N)
    V, F = sim.surface_indexed(G, r)
    assert vertices_match(V, Vg, sha, nv)
    assert len(F) == nf
    if Fg is not None:
        dx = float(np.float32(1.0 / N))
        vdx = oracle_lib.voxel_dx(N, dx, G)
        counts, _ = oracle_lib.surface_table()
        bad, cubes = cube_loop_mismatches(F, Fg, cube_masks(sim.surface_distance(G, r), r, vdx), counts)
        assert cubes > 0 and bad == 0


def test_simulated_body_surface_is_closed(gpu_lib):
    x = _ball(40000, (0.5, 0.5, 0.5), 0.2, 3)
    sim = _sim(x, 48)
    sim.advance(20)
    tris = sim.surface_mesh(96, 3)
    V, F = weld(tris)
    assert edge_balance(F) == 0
    assert enclosed_volume(tris) > (4 / 3) * np.pi * 0.2 ** 3


def test_empty_and_invalid(gpu_lib):
    from mpm_gb300 import _lib

    sim = _sim(np.zeros((0, 3), np.float32))
    assert sim.surface_mesh(16, 2).shape == (0, 3, 3)
    V, F = sim.surface_indexed(16, 2)
    assert V.shape == (0, 3) and F.shape == (0, 3)
    f = sim.surface_distance(16, 2)
    assert np.all(f == np.float32(3 * (1.0 / 16)))
    with pytest.raises(_lib.MpmError):
        sim.surface_mesh(1, 2)
    with pytest.raises(_lib.MpmError):
        sim.surface_distance(16, -1)


def test_mesh_builder_writes_obj(gpu_lib, tmp_path):
    from mpm_gb300.mesh_builder import MeshBuilder

    sim = _sim(_ball(20000, (0.4, 0.5, 0.6), 0.15, 4), 32)
    p = tmp_path / "mesh_00000.obj"
    faces = MeshBuilder(64, 2).computeMesh(str(p), sim)
    text = p.read_text()
    assert faces > 500 and text.count("\nf ") + text.startswith("f ") == faces
    # the v lines read back to the indexed mesh's doubles exactly
    V, F = sim.surface_indexed(64, 2)
    v = np.array([[float(t) for t in l.split()[1:]] for l in text.splitlines() if l.startswith("v ")])
    assert np.array_equal(v, V)


def test_device_outputs_match_host_calls(gpu_lib):
    import ctypes

    from mpm_gb300 import _lib

    sim = _sim(_ball(20000, (0.5, 0.5, 0.5), 0.2, 6), 32)
    tris = sim.surface_mesh(64, 3)
    ptr, n = ctypes.c_void_p(), ctypes.c_int64()
    _lib.check(sim.L.mpm_surface_mesh_device(sim.ctx, 64, 3, ctypes.byref(ptr), ctypes.byref(n)), sim.ctx)
    assert ptr.value and n.value == len(tris)
    _lib.check(sim.L.mpm_surface_distance_device(sim.ctx, 64, 3, ctypes.byref(ptr)), sim.ctx)
    sim.sync()
    assert ptr.value
    # the device calls leave the host calls' results unchanged
    assert np.array_equal(sim.surface_mesh(64, 3), tris)
    V, F = sim.surface_indexed(64, 3)
    vp, fp, nv, nf = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_int64()
    _lib.check(sim.L.mpm_surface_mesh_indexed_device(sim.ctx, 64, 3, ctypes.byref(vp), ctypes.byref(fp),
                                                     ctypes.byref(nv), ctypes.byref(nf)), sim.ctx)
    sim.sync()
    assert vp.value and fp.value and nv.value == len(V) and nf.value == len(F) == len(tris)
