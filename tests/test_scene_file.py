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
