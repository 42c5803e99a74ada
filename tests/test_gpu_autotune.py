"""GPU tests of the fused kernel's launch shapes and of the autotuner (mpm_autotune).

Every launch shape the autotuner can pick (steps per warp, 4/6/12 warps per CTA, the three
G2P tile boxes) must give the oracle's result: one substep within the 1e-5 parity bar of
tests/test_gpu_parity.py.  The search itself runs on a small scene with a bounded budget;
the shape it picks is then checked the same way, and the cache file makes a second search
for the same workload class a lookup."""
import json

import numpy as np
import pytest

from helpers import compare_states

pytestmark = pytest.mark.gpu


def oracle_after(oracle_lib, cfg, nsteps):
    mats = [m.derived() for m in cfg["materials"]]
    out, _, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, nsteps, np.float32)
    return out


def scenes_under_test():
    from mpm_gb300 import scenes

    return {
        "liquid": scenes.config_liquid(n=150_000, seed=31),
        "snow": scenes.config_snow(n=80_000, seed=32, N=48),
        "sparse_elastic": scenes.config_elastic(n=6_000, seed=33, N=32),
    }


SHAPES = [(1, 12, 1), (2, 4, 1), (4, 6, 1), (2, 12, 2), (2, 12, 3), (8, 12, 3)]


@pytest.mark.parametrize("name", ["liquid", "snow", "sparse_elastic"])
@pytest.mark.parametrize("spw,warps,box", SHAPES)
def test_every_launch_shape_matches_oracle(gpu_lib, oracle_lib, name, spw, warps, box):
    from mpm_gb300.simulation import Simulation

    cfg = scenes_under_test()[name]
    with Simulation.from_config(cfg) as sim:
        sim.set_tuning(spw, warps, box)
        sim.upload(cfg["state"])
        sim.advance(3)
        out = sim.syncDevice()
    ref = oracle_after(oracle_lib, cfg, 3)
    errs = compare_states(out, ref, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs


def test_set_tuning_rejects_invalid_shapes(gpu_lib):
    from mpm_gb300 import _lib, scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=1000, seed=34)
    with Simulation.from_config(cfg) as sim:
        L, ctx = sim.L, sim.ctx
        assert L.mpm_set_tuning(ctx, 0, 8, 0) == 1  # 8 warps is not a CTA size
        assert L.mpm_set_tuning(ctx, 0, 0, 4) == 1  # no box 4
        assert L.mpm_set_tuning(ctx, 0, 4, _lib.TILE_4x4x4) == 1  # boxes 2 and 3 run with 12 warps
        assert L.mpm_set_tuning(ctx, 300, 0, 0) == 1
        assert L.mpm_set_tuning(ctx, 4, 12, _lib.TILE_4x6x6) == 0
        from mpm_gb300 import autotune

        cur = autotune.current(sim)
        assert (cur["steps_per_warp"], cur["warps_per_cta"], cur["tile_box"]) == (4, 12, "4x6x6")


def test_autotune_search_cache_and_parity(gpu_lib, oracle_lib, tmp_path):
    """A bounded search (16 timed substeps per candidate) on a 150k-particle liquid scene,
    with the sort interval; the caller's state is untouched by the search; the chosen shape
    runs within the parity bar; the cache answers the second search for the same class
    without measuring and the same shape comes back; another class is measured."""
    from mpm_gb300 import autotune, scenes
    from mpm_gb300.simulation import Simulation

    cache = str(tmp_path / "tuning.json")
    cfg = scenes_under_test()["liquid"]
    with Simulation.from_config(cfg) as sim:
        sim.upload(cfg["state"])
        before = sim.syncDevice()
        t = autotune.tune(sim, cache, tune_sort_interval=True, budget_substeps=16)
        assert not t["from_cache"] and t["candidates"] >= 10 and t["us_per_substep"] > 0
        assert t["sort_interval"] in (4, 8, 16, 32, 64)
        after = sim.syncDevice()
        for k in ("x", "v", "C", "Jp"):
            assert np.array_equal(before[k], after[k]), k  # the search ran on a copy
        assert autotune.current(sim)["steps_per_warp"] == t["steps_per_warp"]
        sim.advance(2)
        out = sim.syncDevice()
    ref = oracle_after(oracle_lib, cfg, 2)
    errs = compare_states(out, ref, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, (t, errs)

    entries = json.load(open(cache))["entries"]
    assert len(entries) == 1 and entries[0]["steps_per_warp"] == t["steps_per_warp"]
    cfg2 = scenes.config_liquid(n=150_000, seed=35)  # same class: layout, N, count, materials
    with Simulation.from_config(cfg2) as sim:
        sim.upload(cfg2["state"])
        t2 = autotune.tune(sim, cache, tune_sort_interval=True, budget_substeps=16)
    assert t2["from_cache"] and t2["candidates"] == 0
    assert {k: t2[k] for k in ("steps_per_warp", "warps_per_cta", "tile_box", "sort_interval")} == \
        {k: t[k] for k in ("steps_per_warp", "warps_per_cta", "tile_box", "sort_interval")}
    cfg3 = scenes_under_test()["snow"]
    with Simulation.from_config(cfg3) as sim:
        sim.upload(cfg3["state"])
        t3 = autotune.tune(sim, cache, budget_substeps=8)
        assert not t3["from_cache"]
        sim.advance(1)
        out = sim.syncDevice()
    ref = oracle_after(oracle_lib, cfg3, 1)
    errs = compare_states(out, ref, cfg3["params"], cfg3["state"])
    assert max(errs.values()) < 1e-5, (t3, errs)
    assert len(json.load(open(cache))["entries"]) == 2


def test_batch_autotune_picks_a_range_size_and_keeps_parity(gpu_lib, oracle_lib, tmp_path):
    """mpm_batch_autotune times the batched kernel's range sizes on a copy of the batch
    (the batch's own particles do not change), applies the fastest, stores it in the
    cache (a second search is a lookup), and the tuned batch still matches the oracle per
    scene."""
    from mpm_gb300 import autotune, scenes
    from mpm_gb300.batch import Batch

    scs = scenes.config_batched(nscenes=8, seed=21, count_range=(2_000, 30_000))
    cache = str(tmp_path / "tuning.json")
    with Batch(scs, sort_interval=4) as b:
        b.upload([s["state"] for s in scs])
        before = b.download()
        t = autotune.tune_batch(b, cache, budget_substeps=12)
        assert t["steps_per_warp"] in (1, 2, 4, 8, 16) and not t["from_cache"] and t["candidates"] == 5
        assert t["us_per_substep"] > 0
        assert autotune.current_batch(b)["steps_per_warp"] == t["steps_per_warp"]
        after = b.download()
        for k in before:
            assert np.array_equal(before[k], after[k]), k
        t2 = autotune.tune_batch(b, cache, budget_substeps=12)
        assert t2["from_cache"] and t2["steps_per_warp"] == t["steps_per_warp"]
        b.advance(3)
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        ref = oracle_after(oracle_lib, {"state": sc["state"], "params": sc["params"], "materials": [sc["material"]]}, 3)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert max(errs.values()) < 2e-5, (sc["params"]["N"], sc["material"].name, errs)
    entries = json.load(open(cache))["entries"]
    assert any(e["class"].startswith("batch scenes=8") for e in entries)


@pytest.mark.parametrize("spw", [1, 16])
def test_batch_range_sizes_match_oracle(gpu_lib, oracle_lib, spw):
    """Any range size gives the oracle's result (ranges only split the work)."""
    from mpm_gb300 import scenes
    from mpm_gb300.batch import Batch

    scs = scenes.config_batched(nscenes=6, seed=22, count_range=(1_500, 20_000))
    with Batch(scs, sort_interval=2) as b:
        b.set_steps_per_warp(spw)
        b.upload([s["state"] for s in scs])
        b.advance(3, graph=True)
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        ref = oracle_after(oracle_lib, {"state": sc["state"], "params": sc["params"], "materials": [sc["material"]]}, 3)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert max(errs.values()) < 2e-5, (spw, sc["params"]["N"], errs)


def test_batch_autotune_sort_interval(gpu_lib, oracle_lib):
    """With the sort interval among the knobs, the batch tuner also times intervals of 8, 12,
    16 and 24 substeps (replays of 48) and applies the fastest; the tuned batch still
    matches the oracle per scene."""
    from mpm_gb300 import autotune, scenes
    from mpm_gb300.batch import Batch

    scs = scenes.config_batched(nscenes=6, seed=23, count_range=(2_000, 20_000))
    with Batch(scs, sort_interval=4) as b:
        b.upload([s["state"] for s in scs])
        t = autotune.tune_batch(b, None, budget_substeps=6, tune_sort_interval=True)
        assert t["candidates"] == 10 and not t["from_cache"]
        assert t["sort_interval"] in (4, 8, 12, 16, 24)
        assert autotune.current_batch(b)["sort_interval"] == t["sort_interval"]
        b.advance(3, graph=True)
        outs = b.split(b.download())
    for sc, out in zip(scs, outs):
        ref = oracle_after(oracle_lib, {"state": sc["state"], "params": sc["params"], "materials": [sc["material"]]}, 3)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        assert max(errs.values()) < 2e-5, (t, sc["params"]["N"], errs)
