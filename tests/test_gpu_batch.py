"""GPU tests of the batched-scenes path: every scene of a batch must evolve exactly as
it would alone (same oracle parity bar as the plain path), with and without the
replayed CUDA graph."""
import numpy as np
import pytest

from helpers import compare_states

pytestmark = pytest.mark.gpu


def small_batch(seed=0, nscenes=10):
    from mpm_gb300 import scenes

    return scenes.config_batched(nscenes=nscenes, seed=seed, count_range=(1_500, 20_000))


def oracle_scene(oracle_lib, sc, nsteps):
    st = dict(sc["state"])
    out, _, _ = oracle_lib.substep(st, sc["params"], [sc["material"].derived()], nsteps, np.float32)
    return out


def test_batch_matches_oracle_per_scene(gpu_lib, oracle_lib):
    from mpm_gb300.batch import Batch

    scs = small_batch(seed=1)
    with Batch(scs, sort_interval=2) as b:
        b.upload([s["state"] for s in scs])
        b.advance(4)
        b.sync()
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        ref = oracle_scene(oracle_lib, sc, 4)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert max(errs.values()) < 2e-5, (sc["params"]["N"], sc["material"].name, errs)


def test_batch_sorts_keep_particles_outside_the_domain(gpu_lib, oracle_lib):
    """The batch's sorts move only what the next fused launch reads back for particles
    inside their scene's domain; particles completely outside it (each scene with its own
    N) keep their whole state through sorts before every substep, in the launched and the
    replayed-graph runs."""
    from helpers import FIELDS
    from mpm_gb300.batch import Batch

    scs = small_batch(seed=4, nscenes=6)
    rng = np.random.default_rng(5)
    idx = []
    for sc in scs:
        st = sc["state"]
        k = rng.choice(st["x"].shape[0], 50, replace=False)
        st["x"][k] = rng.uniform(1.3, 1.9, (50, 3)).astype(np.float32)  # base cells past N
        st["v"][k] = rng.standard_normal((50, 3)).astype(np.float32)
        st["C"][k] = rng.standard_normal((50, 3, 3)).astype(np.float32)
        st["F"][k] += (0.01 * rng.standard_normal((50, 3, 3))).astype(np.float32)
        idx.append(k)
    for graph in (False, True):
        with Batch(scs, sort_interval=1) as b:
            b.upload([s["state"] for s in scs])
            b.advance(4, graph=graph)
            outs = b.split(b.download())
        for sc, out, k in zip(scs, outs, idx):
            for f in FIELDS:
                assert np.array_equal(out[f][k], sc["state"][f][k]), (graph, f)
            if not graph:
                ref = oracle_scene(oracle_lib, sc, 4)
                errs = compare_states(out, ref, sc["params"], sc["state"])
                assert max(errs.values()) < 2e-5, (sc["params"]["N"], sc["material"].name, errs)


def test_batch_matches_single_scene_contexts(gpu_lib):
    from mpm_gb300.batch import Batch
    from mpm_gb300.simulation import Simulation

    scs = small_batch(seed=2)
    with Batch(scs, sort_interval=3) as b:
        b.upload([s["state"] for s in scs])
        b.advance(6)
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        with Simulation(materials=[sc["material"]], sort_interval=3, **sc["params"]) as sim:
            sim.upload(sc["state"])
            sim.advance(6)
            ref = sim.syncDevice()
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert max(errs.values()) < 2e-5, errs


def test_batch_graph_replay_matches_launches(gpu_lib):
    """Two graph replays of 5 substeps equal 10 launched substeps (the graph re-sorts at
    the start of each replay; sorting does not change results beyond rounding)."""
    from mpm_gb300.batch import Batch

    scs = small_batch(seed=3, nscenes=12)
    states = [s["state"] for s in scs]
    with Batch(scs, sort_interval=5) as b:
        b.upload(states)
        b.advance(10)
        ref = b.download()
    with Batch(scs, sort_interval=5) as b:
        b.upload(states)
        b.advance(5, graph=True)
        b.advance(5, graph=True)
        b.sync()
        out = b.download()
        b.advance(5, graph=True)  # a third replay from another phase runs too
        b.sync()
    p = scs[0]["params"]
    errs = compare_states(out, ref, p, {"v": np.concatenate([s["v"] for s in states])})
    assert max(errs.values()) < 2e-5, errs


@pytest.mark.parametrize("interval", [4, 6])
def test_batch_graph_sorts_at_the_interval(gpu_lib, interval):
    """A replayed graph sorts before its first substep and then every sort_interval
    substeps, as launched substeps do: 12 replayed substeps hold 3 sorts (an odd count, which
    swaps the particle buffers) with interval 4 and 2 with interval 6. Two replays equal 24
    launched substeps to rounding."""
    from mpm_gb300.batch import Batch

    scs = small_batch(seed=6, nscenes=8)
    states = [s["state"] for s in scs]
    with Batch(scs, sort_interval=interval) as b:
        b.upload(states)
        b.advance(24)
        ref = b.download()
    with Batch(scs, sort_interval=interval) as b:
        b.upload(states)
        l0 = b.launches
        b.advance(12, graph=True)
        b.advance(12, graph=True)
        b.sync()
        out = b.download()
        assert b.launches > l0
    p = scs[0]["params"]
    errs = compare_states(out, ref, p, {"v": np.concatenate([s["v"] for s in states])})
    assert max(errs.values()) < 2e-5, errs


def test_batch_long_run_clears_grids(gpu_lib, oracle_lib):
    """40 substeps with the sparse grid clearing: the batch stays on the single-scene
    trajectory (stale grid data would show up as drift)."""
    from mpm_gb300.batch import Batch

    scs = small_batch(seed=4, nscenes=6)
    with Batch(scs, sort_interval=8) as b:
        b.upload([s["state"] for s in scs])
        b.advance(40, graph=False)
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        ref = oracle_scene(oracle_lib, sc, 40)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert errs["x"] < 1e-5 and errs["v"] < 1e-3, errs


def test_full_batched_config_runs(gpu_lib):
    """The 256-scene configuration: one graph of 50 substeps runs, mass stays put."""
    from mpm_gb300 import scenes
    from mpm_gb300.batch import Batch

    scs = scenes.config_batched(nscenes=256, seed=0)
    with Batch(scs, sort_interval=16) as b:
        b.upload([s["state"] for s in scs])
        b.advance(50, graph=True)
        b.sync()
        out = b.download()
    assert np.isfinite(out["x"]).all() and np.isfinite(out["v"]).all()
    x0 = np.concatenate([s["state"]["x"] for s in scs])
    assert np.abs(out["x"] - x0).max() < 0.05  # 50 substeps at dt 1e-4 move particles by < 1 cell
