"""Long-run parity of the CUDA substep against the FP64 oracle at the full workload sizes.

One substep agrees with the oracle to 1e-5 (tests/test_gpu_parity.py); these tests run the
liquid and snow workloads for their full substep counts and the batched and differentiable
workloads at their full sizes.

Bounds of the long runs (GPU FP32 against the FP64 oracle, sampled every 100 substeps):
  * total mass: the GPU's post-P2G grid mass equals m n to 1e-6 relative (float atomics;
    every particle stays inside the grid), the oracle's to 1e-10;
  * momentum (sum of m v) and kinetic energy: within 1e-4 relative;
  * mean Jp (liquid: J; snow: the plastic volume ratio): within 1e-4 absolute;
  * after the last block, the particle fields x within 1e-5 and v within 1e-3 relative
    (norm-wise, tests/helpers.py).
The CPU oracle in FP32 stays within 2e-5 (momentum, energy, mean Jp, v) and 8e-7 (x) of
the FP64 oracle over the same runs at a tenth of the particles: the bounds leave about a
factor of 5 for the GPU's different summation order (float atomics, cell sort every 16
substeps).
"""
import numpy as np
import pytest

from helpers import compare_states

pytestmark = pytest.mark.gpu


def aggregates(st, m):
    v = st["v"].astype(np.float64)
    return m * v.sum(0), 0.5 * m * float((v ** 2).sum()), float(st["Jp"].astype(np.float64).mean())


def long_run(oracle_lib, cfg, total, block=100):
    """Advances the GPU (FP32, cell sort as configured) and the FP64 oracle side by side
    and checks the bounds above after every block of substeps."""
    from mpm_gb300.simulation import Simulation

    mats = [m.derived() for m in cfg["materials"]]
    m = float(mats[0]["particle_mass"])
    n = cfg["state"]["x"].shape[0]
    ref = {k: np.array(v, np.float64) if k != "mat" else v for k, v in cfg["state"].items()}
    log = []
    with Simulation.from_config(cfg) as sim:
        sim.upload(cfg["state"])
        for k in range(total // block):
            sim.advance(block)
            out = sim.syncDevice()
            grid = sim.get_grid(0)
            ref, g_ref, _ = oracle_lib.substep(ref, cfg["params"], mats, block, np.float64, want_grids=True)
            p_gpu, ke_gpu, j_gpu = aggregates(out, m)
            p_ref, ke_ref, j_ref = aggregates(ref, m)
            mass_gpu = float(grid[..., 3].astype(np.float64).sum())
            mass_ref = float(g_ref[..., 3].sum())
            step = (k + 1) * block
            log.append((step, np.linalg.norm(p_gpu - p_ref) / np.linalg.norm(p_ref), abs(ke_gpu - ke_ref) / ke_ref,
                        abs(j_gpu - j_ref)))
            assert abs(mass_ref - m * n) <= 1e-10 * m * n, (step, mass_ref, m * n)
            assert abs(mass_gpu - m * n) <= 1e-6 * m * n, (step, mass_gpu, m * n)
            assert np.linalg.norm(p_gpu - p_ref) <= 1e-4 * np.linalg.norm(p_ref), (step, p_gpu, p_ref)
            assert abs(ke_gpu - ke_ref) <= 1e-4 * ke_ref, (step, ke_gpu, ke_ref)
            assert abs(j_gpu - j_ref) <= 1e-4, (step, j_gpu, j_ref)
    for step, dp, dke, dj in log:
        print(f"{cfg['name']} substep {step}: momentum {dp:.2e} kinetic energy {dke:.2e} mean Jp {dj:.2e}")
    errs = compare_states(out, ref, cfg["params"], ref)
    print(cfg["name"], "fields after the run:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert errs["x"] < 1e-5, errs
    assert errs["v"] < 1e-3, errs
    return log, errs


def test_liquid_1000_substeps(gpu_lib, oracle_lib):
    """The liquid workload in full: 1,000,000 particles, N = 32, cell sort every 16
    substeps, 1000 substeps (0.1 s of simulated time)."""
    from mpm_gb300 import scenes

    cfg = scenes.config_liquid()
    assert cfg["params"]["sort_interval"] == 16
    long_run(oracle_lib, cfg, 1000)


def test_snow_500_substeps(gpu_lib, oracle_lib):
    """The snow workload in full: 500,000 particles in two spheres, N = 64, SVD plasticity
    with hardening, 500 substeps; mean Jp tracks the plastic compression."""
    from mpm_gb300 import scenes

    cfg = scenes.config_snow()
    long_run(oracle_lib, cfg, 500)


def test_full_batched_config_per_scene_parity(gpu_lib, oracle_lib):
    """The batched workload in full (256 scenes, 2k-200k particles, N in {16, 32, 64},
    elastic, liquid and snow): every scene after one batched substep matches the FP32
    oracle at 1e-5, and a 50-substep replayed graph matches each scene advanced alone
    through its own context at the long-run bounds (x 1e-5, v 1e-3)."""
    from mpm_gb300 import scenes
    from mpm_gb300.batch import Batch
    from mpm_gb300.simulation import Simulation

    scs = scenes.config_batched(nscenes=256, seed=0)
    assert len(scs) == 256 and {s["params"]["N"] for s in scs} == {16, 32, 64}
    with Batch(scs, sort_interval=16) as b:
        b.upload([s["state"] for s in scs])
        b.advance(1)
        b.sync()
        one = b.split(b.download())
    worst = 0.0
    for sc, out in zip(scs, one):
        ref, _, _ = oracle_lib.substep(sc["state"], sc["params"], [sc["material"].derived()], 1, np.float32)
        errs = compare_states(out, ref, sc["params"], sc["state"])
        worst = max(worst, max(errs.values()))
        assert max(errs.values()) < 1e-5, (sc["name"], sc["params"]["N"], sc["material"].name, errs)

    with Batch(scs, sort_interval=16) as b:
        b.upload([s["state"] for s in scs])
        b.advance(50, graph=True)
        b.sync()
        fifty = b.split(b.download())
    for sc, out in zip(scs, fifty):
        with Simulation(materials=[sc["material"]], sort_interval=16, **sc["params"]) as sim:
            sim.upload(sc["state"])
            sim.advance(50)
            alone = sim.syncDevice()
        errs = compare_states(out, alone, sc["params"], sc["state"])
        assert errs["x"] < 1e-5 and errs["v"] < 1e-3, (sc["name"], errs)
