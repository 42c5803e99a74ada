"""GPU tests of particle export (mpm_export_*, ParticleWriter) and headless rendering
(mpm_render_*): the packed .bgeo records and files against the oracle's restatement of the
reference's Partio file (include/particle_writer.h:19-43) in active-list order, the copy
overlapping later substeps, and the rasterised image against the oracle rasteriser."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(n=50000, N=32, seed=0, liquid=False):
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    rng = np.random.default_rng(seed)
    x = (0.2 + 0.5 * rng.random((n, 3))).astype(np.float32)
    v = rng.normal(scale=0.3, size=(n, 3)).astype(np.float32)
    sim = Simulation(dt=1e-4, N=N, sort_interval=4)
    sim.set_materials([M.liquid(1.0 / n) if liquid else M.snow(1.0 / n)])
    sim.upload({"x": x, "v": v})
    return sim


@pytest.mark.parametrize("liquid", [False, True])
def test_records_match_oracle_in_active_order(gpu_lib, liquid):
    from mpm_gb300 import particle_writer as W

    from oracle import export_oracle as E

    sim = _sim(liquid=liquid)
    sim.advance(9)  # cell-sorted twice: device order differs from the active-list order
    st = sim.download(("x", "v"))
    W.export_records(sim, 0)
    assert W.records_bytes(sim, 0) == E.bgeo_records(st["x"], st["v"])


def test_export_copy_overlaps_later_substeps(gpu_lib):
    from mpm_gb300 import particle_writer as W

    from oracle import export_oracle as E

    sim = _sim()
    sim.advance(3)
    before = sim.download(("x", "v"))
    W.export_records(sim, 1)
    sim.advance(5)  # enqueued behind the packing, alongside the copy
    assert W.records_bytes(sim, 1) == E.bgeo_records(before["x"], before["v"])
    after = sim.download(("x", "v"))
    assert not np.array_equal(after["x"], before["x"])


def test_writers_write_reference_files(gpu_lib, tmp_path):
    from mpm_gb300.particle_writer import AsyncParticleWriter, ParticleWriter

    from oracle import export_oracle as E

    sim = _sim(20000)
    p0 = tmp_path / "particles_0.bgeo"
    ParticleWriter().writeParticles(str(p0), sim)
    st = sim.download(("x", "v"))
    assert p0.read_bytes() == E.bgeo_file(st["x"], st["v"])
    frames = []
    with AsyncParticleWriter(compress=True) as w:
        for f in range(5):
            st = sim.download(("x", "v"))
            frames.append(st)
            w.submit(str(tmp_path / f"particles_{f + 1}.bgeo"), sim)
            sim.advance(4)
    for f, st in enumerate(frames):
        parsed = E.parse_bgeo((tmp_path / f"particles_{f + 1}.bgeo").read_bytes())
        ref = E.parse_bgeo(E.bgeo_file(st["x"], st["v"]))
        assert np.array_equal(parsed["records"], ref["records"]) and parsed["tail"] == b"\x00\xff"


def test_export_of_objects_and_empty_context(gpu_lib):
    from mpm_gb300 import _lib
    from mpm_gb300 import materials as M
    from mpm_gb300 import particle_writer as W
    from mpm_gb300.scene_file import SceneObject
    from mpm_gb300.simulation import Simulation

    from oracle import export_oracle as E

    sim = Simulation(dt=1e-4, N=32, sort_interval=2)
    sim.set_materials([M.elastic(1e-5)])
    sim.upload({"x": np.zeros((0, 3), np.float32)})
    assert W.export_records(sim, 0) == 0 and W.records_bytes(sim, 0) == b""
    sim.add_object(SceneObject(shape=_lib.SHAPE_SPHERE, size=0.2, position=(0.3, 0.3, 0.3), seed=4))
    sim.add_object(SceneObject(shape=_lib.SHAPE_BOX, size=0.1, position=(0.6, 0.5, 0.5), seed=5,
                               lifetime_begin=2.5e-4))
    sim.advance(5)
    st = sim.download(("x", "v"))
    W.export_records(sim, 0)
    assert W.records_bytes(sim, 0) == E.bgeo_records(st["x"], st["v"])


def test_render_matches_oracle(gpu_lib):
    from mpm_gb300.renderer import Renderer

    from oracle import export_oracle as E

    sim = _sim(30000)
    sim.advance(6)
    x = sim.download(("x",))["x"]
    r = Renderer()
    assert np.array_equal(r.positions(sim), E.positions(x))
    img = r.render(sim)
    assert np.array_equal(img, E.render_points(x))
    assert (img[..., 0] == 150).sum() > 1000
    # another size and point size, and particles outside the clip volume
    x2 = np.concatenate([x, np.array([[-0.2, 0.5, 0.5], [0.5, 1.3, 0.5], [0.0, 0.0, 0.5]], np.float32)])
    sim.upload({"x": x2})
    r2 = Renderer(320, 200, point_size=3.0)
    assert np.array_equal(r2.render(sim), E.render_points(x2, 320, 200, 3.0))
