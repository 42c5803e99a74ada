"""CPU tests of the scene objects row: the reference-format TOML reader, the OBJ
reader, and the oracle's restatement of the rejection sampler (the checker of the GPU
seeder)."""
import os

import numpy as np
import pytest

from helpers import icosphere, write_obj

SCENE = """
[[material]]
name = "snow"
density = 700
E = 1.4e5
Nu = 0.2
hardening = 10
plast_clamp_lower = 0.975
plast_clamp_higher = 1.0075

[[material]]
name = "jelly"
density = 300

[[object]]
material = "jelly"
mesh = "cube.obj"
size = 0.3
position = [0.35, 0.5, 0.35]
velocity = [0.0, -1.0, 0.0]
lifetime_begin = 2.0

[[object]]
material = "snow"
mesh = "sphere.obj"
size = 0.2
position = [0.4, 0.1, 0.4]
velocity = [0.0, 0.0, 0.0]

[[object]]
material = "snow"
mesh = "ico.obj"
size = 0.25
position = [0.1, 0.6, 0.1]
velocity = [1.0, 0.0, 0.0]
lifetime_end = 3.5
"""


def test_load_scene_reference_format(tmp_path):
    pytest.importorskip("tomllib")
    from mpm_gb300 import _lib
    from mpm_gb300.scene_file import FOREVER, load_scene

    os.makedirs(tmp_path / "meshes")
    V, F = icosphere(1)
    write_obj(tmp_path / "meshes" / "ico.obj", V, F)
    (tmp_path / "s.toml").write_text(SCENE)
    mats, objs = load_scene(str(tmp_path / "s.toml"), particle_count=200000)
    assert [m.name for m in mats] == ["snow", "jelly"]
    # MMSnow defaults of src/main.cu:35-43 for the fields jelly leaves out
    assert mats[1].density == 300 and mats[1].E == 1.4e5 and mats[1].nu == 0.2 and mats[1].hardening == 10.0
    assert mats[1].clamp_lo == 0.975 and mats[1].clamp_hi == 1.0075
    assert all(m.particle_volume == 1.0 / 200000 for m in mats)
    assert [o.shape for o in objs] == [_lib.SHAPE_BOX, _lib.SHAPE_SPHERE, _lib.SHAPE_MESH]
    assert [o.material for o in objs] == [1, 0, 0]
    assert objs[0].lifetime_begin == 2.0 and objs[0].lifetime_end == FOREVER
    assert objs[2].lifetime_end == 3.5 and objs[2].velocity == (1.0, 0.0, 0.0)
    assert objs[2].triangles.shape == F.shape


def test_read_obj_fans_polygons(tmp_path):
    from mpm_gb300.scene_file import read_obj

    p = tmp_path / "q.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    V, F = read_obj(str(p))
    assert V.shape == (4, 3) and F.tolist() == [[0, 1, 2], [0, 2, 3]]
    stub = tmp_path / "lfs.obj"
    stub.write_text("version https://git-lfs.github.com/spec/v1\noid sha256:00\nsize 1\n")
    with pytest.raises(ValueError):
        read_obj(str(stub))


def test_oracle_sampler_density_and_inside(oracle_lib):
    """src/mpm.cu:369-371: candidates = u32(density x box volume); the kept count of a
    sphere follows the binomial law around density x sphere volume."""
    dens, size = 400000, 0.2
    x = oracle_lib.seed_object(1, size, (0.3, 0.3, 0.3), seed=11, density=dens)
    cand = int(dens * size ** 3)
    p = np.pi / 6.0
    assert abs(len(x) - cand * p) < 5 * np.sqrt(cand * p * (1 - p))
    c = np.array([0.4, 0.4, 0.4])
    assert np.all(np.linalg.norm(x.astype(np.float64) - c, axis=1) < size / 2 + 1e-6)
    # reproducible and seed-dependent
    assert np.array_equal(x, oracle_lib.seed_object(1, size, (0.3, 0.3, 0.3), seed=11, density=dens))
    assert not np.array_equal(x[:10], oracle_lib.seed_object(1, size, (0.3, 0.3, 0.3), seed=12, density=dens)[:10])


def mesh_volume(V, F):
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def test_oracle_mesh_parity_matches_the_mesh_volume(oracle_lib):
    """Ray parity on a closed icosphere: every kept point lies in the mesh's
    circumscribed ball, and the kept count follows density x mesh volume."""
    V, F = icosphere(3)
    dens, size, pos = 200000, 0.3, np.array([0.2, 0.2, 0.2])
    xm = oracle_lib.seed_object(2, size, pos, seed=5, density=dens, vertices=V, triangles=F).astype(np.float64)
    Vd = V.astype(np.float64)
    lo, hi = Vd.min(0), Vd.max(0)
    scale = size / (hi - lo).max()
    Vs = (Vd - lo) * scale + pos
    c = (Vs.min(0) + Vs.max(0)) / 2
    assert np.linalg.norm(xm - c, axis=1).max() <= np.linalg.norm(Vs - c, axis=1).max() * (1 + 1e-6)
    cand = int(dens * np.prod(Vs.max(0) - Vs.min(0)))
    p = mesh_volume(Vs, F) / np.prod(Vs.max(0) - Vs.min(0))
    assert abs(len(xm) - cand * p) < 5 * np.sqrt(cand * p * (1 - p)), (len(xm), cand * p)


def _winding_numbers(Vs, F, P):
    """Generalized winding numbers of points P, as numpy float64 solid angles."""
    a, b, c = (Vs[F[:, k]][None, :, :] - P[:, None, :] for k in range(3))
    la, lb, lc = (np.linalg.norm(x, axis=2) for x in (a, b, c))
    det = np.einsum("ptj,ptj->pt", a, np.cross(b, c))
    den = la * lb * lc + np.einsum("ptj,ptj->pt", b, c) * la + np.einsum("ptj,ptj->pt", c, a) * lb + \
        np.einsum("ptj,ptj->pt", a, b) * lc
    return (np.arctan2(det, den) / (2 * np.pi)).sum(1)


def _splitmix64(z):
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _candidates(seed, lo, rng, n):
    """Candidates 0..n-1 of the rejection sampler: float(lo + u range), u from SplitMix64 of
    seed + 3 i + axis with 53 bits."""
    i = np.arange(n, dtype=np.uint64)
    out = np.empty((n, 3), np.float32)
    for c in range(3):
        u = (_splitmix64(np.uint64(seed) + np.uint64(3) * i + np.uint64(c)) >> np.uint64(11)).astype(np.float64) \
            * (1.0 / 9007199254740992.0)
        out[:, c] = (lo[c] + u * rng[c]).astype(np.float32)
    return out


def _placed(V, size, pos):
    Vd = V.astype(np.float32)
    lo, hi = Vd.min(0), Vd.max(0)
    scale = np.float32(size) / (hi - lo).max()
    return (Vd * scale + (np.asarray(pos, np.float32) - scale * lo)).astype(np.float32)


def test_oracle_winding_number_inside_test(oracle_lib):
    """The oracle's winding-number test (inside_test = 1): on a closed mesh it keeps the same
    particles as ray parity; on a mesh with a hole and on two overlapping spheres its kept
    points are those of an independent numpy winding number above 1/2, among the candidates of
    ray parity's run (kept or not)."""
    from helpers import icosphere, open_icosphere, two_spheres

    dens, size, pos = 60000, 0.3, (0.2, 0.2, 0.2)
    V, F = icosphere(2)
    ray = oracle_lib.seed_object(2, size, pos, seed=7, density=dens, vertices=V, triangles=F)
    wind = oracle_lib.seed_object(2, size, pos, seed=7, density=dens, vertices=V, triangles=F, inside_test=1)
    assert len(ray) > 300 and np.array_equal(ray, wind)
    for V, F in (open_icosphere(2), two_spheres(2)):
        Vs = _placed(V, size, pos)
        lo, hi = Vs.min(0).astype(np.float64), Vs.max(0).astype(np.float64)
        cand = _candidates(7, lo, hi - lo, int(dens * np.prod(hi - lo)))
        w = _winding_numbers(Vs.astype(np.float64), F, cand.astype(np.float64))
        wind = oracle_lib.seed_object(2, size, pos, seed=7, density=dens, vertices=V, triangles=F, inside_test=1)
        assert np.array_equal(wind, cand[w > 0.5])
    ray = oracle_lib.seed_object(2, size, pos, seed=7, density=dens, vertices=V, triangles=F)
    assert len(wind) > len(ray) * 1.2  # the overlap of the two spheres is inside only by the winding number


def test_open_meshes_use_the_winding_number():
    from helpers import icosphere, open_icosphere, two_spheres

    from mpm_gb300.scene_file import is_closed

    assert is_closed(icosphere(2)[1]) and is_closed(two_spheres(2)[1])
    assert not is_closed(open_icosphere(2)[1])
    F = icosphere(1)[1]
    assert not is_closed(F[:, [0, 2, 1]][:1].tolist() + F[1:].tolist())  # one flipped triangle
