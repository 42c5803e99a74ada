"""GPU parity tests: the CUDA substep (through the C ABI) against the CPU oracle.

Bars (written per test):
  * one substep, FP32 oracle vs GPU: particle x, v, C, F, Jp and the grid after P2G
    (mass and momentum) within 1e-5 relative (norm-wise, with the field scale of
    tests/helpers.py as floor for fields that are zero up to rounding);
  * the same against the FP64 oracle: within 1e-4 (FP32 rounding of the whole step);
  * multi-substep runs: trajectories of total mass, momentum and kinetic energy.
"""
import numpy as np
import pytest

from helpers import compare_states, rel_err

pytestmark = pytest.mark.gpu


def run_gpu(cfg, nsteps, want_grid=False, **over):
    from mpm_gb300.simulation import Simulation

    with Simulation.from_config(cfg, **over) as sim:
        sim.upload(cfg["state"])
        sim.advance(nsteps)
        out = sim.syncDevice()
        grids = (sim.get_grid(0), sim.get_grid(1)) if want_grid else (None, None)
    return out, grids


def run_oracle(oracle_lib, cfg, nsteps, dtype, params=None):
    mats = [m.derived() for m in cfg["materials"]]
    return oracle_lib.substep(cfg["state"], params or cfg["params"], mats, nsteps, dtype, want_grids=True)


def configs():
    from mpm_gb300 import scenes

    return {
        "elastic_10k_N16": lambda: scenes.config_elastic(),
        "liquid_1M_N32": lambda: scenes.config_liquid(),
        "snow_500k_N64": lambda: scenes.config_snow(),
        "mixed_20k_N32": lambda: scenes.mixed_scene(),
        "fixed_corotated_100k_N64": lambda: scenes.config_differentiable(),
        # grid sides whose padded extents (N + 5) are not powers of two, and a tiny grid
        "elastic_20k_N37": lambda: scenes.config_elastic(n=20_000, seed=5, N=37),
        "elastic_2k_N5": lambda: _with_params(scenes.config_elastic(n=2_000, seed=6, N=5), boundary_cells=2),
    }


def _with_params(cfg, **params):
    cfg["params"].update(params)
    return cfg


@pytest.mark.parametrize("name", list(configs().keys()))
def test_one_substep_parity(gpu_lib, oracle_lib, name):
    cfg = configs()[name]()
    out, (g_p2g, g_op) = run_gpu(cfg, 1, want_grid=True)
    o32, r_p2g, r_op = run_oracle(oracle_lib, cfg, 1, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs
    # grid after P2G: mass and momentum
    assert rel_err(g_p2g[..., 3], r_p2g[..., 3]) < 1e-5
    assert rel_err(g_p2g[..., :3], r_p2g[..., :3], 1e-12) < 1e-5
    # grid after the op (velocities; mass slot 1 where m > 0)
    assert rel_err(g_op[..., :3], r_op[..., :3], 1e-12) < 1e-5
    assert np.array_equal(g_op[..., 3] == 1.0, r_op[..., 3] == 1.0)
    # against FP64
    o64, q_p2g, _ = run_oracle(oracle_lib, cfg, 1, np.float64)
    errs64 = compare_states(out, o64, cfg["params"], cfg["state"])
    assert max(errs64.values()) < 1e-4, errs64
    assert rel_err(g_p2g[..., 3], q_p2g[..., 3]) < 1e-5


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_boundary_modes(gpu_lib, oracle_lib, mode):
    from mpm_gb300 import scenes

    cfg = scenes.config_snow(n=60_000, seed=3, N=32)
    cfg["params"] = dict(cfg["params"], boundary_mode=mode, boundary_cells=3)
    # push the snow against the floor and a wall so the walls act
    cfg["state"]["x"][:, 1] -= 0.15
    cfg["state"]["v"][:, 0] = -2.0
    out, _ = run_gpu(cfg, 5)
    o32, _, _ = run_oracle(oracle_lib, cfg, 5, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 2e-5, errs


def test_g2p_guard_mode(gpu_lib, oracle_lib):
    """src/mpm.cu:114 reproduced: particles with index > N^3 skip G2P but scatter."""
    from mpm_gb300 import scenes

    cfg = scenes.config_elastic(n=10_000, seed=4, N=16)
    cfg["params"] = dict(cfg["params"], g2p_guard=1)
    out, _ = run_gpu(cfg, 3, sort_interval=1)
    o32, _, _ = run_oracle(oracle_lib, cfg, 3, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs
    lim = 16 ** 3
    assert np.array_equal(out["x"][lim + 1:], cfg["state"]["x"][lim + 1:])


@pytest.mark.parametrize("sort_interval", [0, 1, 3])
def test_sort_does_not_change_results(gpu_lib, oracle_lib, sort_interval):
    from mpm_gb300 import scenes

    cfg = scenes.config_liquid(n=200_000, seed=5)
    out, _ = run_gpu(cfg, 6, sort_interval=sort_interval)
    o32, _, _ = run_oracle(oracle_lib, cfg, 6, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 2e-5, errs


@pytest.mark.parametrize("kind", ["liquid", "snow"])
def test_sort_keeps_particles_outside_the_domain(gpu_lib, oracle_lib, kind):
    """A sort between substeps moves only what the next G2P reads back (x and J, or x, F
    and Jp) for particles inside the domain: their v and C are rewritten by that G2P.
    Particles completely outside the domain skip G2P and keep their whole state, so the
    sort moves all of it; here they carry random v, C (and F) that must come back intact
    after sorts between every substep."""
    from helpers import FIELDS
    from mpm_gb300 import scenes

    cfg = scenes.config_liquid(n=60_000, seed=7) if kind == "liquid" else scenes.config_snow(n=60_000, seed=7, N=32)
    st = cfg["state"]
    rng = np.random.default_rng(8)
    idx = rng.choice(st["x"].shape[0], 500, replace=False)
    st["x"][idx] = rng.uniform(-0.9, -0.3, (500, 3)).astype(np.float32)  # base cells below -3
    st["v"][idx] = rng.standard_normal((500, 3)).astype(np.float32)
    st["C"][idx] = rng.standard_normal((500, 3, 3)).astype(np.float32)
    if kind == "snow":
        st["F"][idx] += (0.01 * rng.standard_normal((500, 3, 3))).astype(np.float32)
        st["Jp"][idx] = rng.uniform(0.9, 1.1, 500).astype(np.float32)
    out, _ = run_gpu(cfg, 5, sort_interval=1)
    kept = ("x", "v", "C", "Jp") if kind == "liquid" else FIELDS  # the liquid layout stores no F
    for k in kept:
        assert np.array_equal(out[k][idx], st[k][idx]), k
    o32, _, _ = run_oracle(oracle_lib, cfg, 5, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 2e-5, errs


@pytest.mark.parametrize("kind", ["liquid", "snow"])
def test_explicit_sort_moves_the_whole_state(gpu_lib, kind):
    """mpm_sort between calls is followed by no G2P of its own, so it moves every
    component: a download after it returns exactly what the download before it did."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_liquid(n=40_000, seed=3) if kind == "liquid" else scenes.config_snow(n=40_000, seed=3, N=32)
    with Simulation.from_config(cfg, sort_interval=2) as sim:
        sim.upload(cfg["state"])
        sim.advance(5)
        before = sim.download()
        sim.sort()
        after = sim.download()
        for k in before:
            assert np.array_equal(before[k], after[k]), k
        sim.advance(3)  # and the run goes on from the sorted state
        assert np.isfinite(sim.download()["x"]).all()


@pytest.mark.parametrize("tuning", [(1,), (4,), (16,), (8,)])
def test_tuning_variants(gpu_lib, oracle_lib, tuning):
    """Range sizes (steps per warp) give the same result."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_snow(n=100_000, seed=6, N=64)
    with Simulation.from_config(cfg) as sim:
        sim.set_tuning(*tuning)
        sim.upload(cfg["state"])
        sim.advance(2)
        out = sim.syncDevice()
    o32, _, _ = run_oracle(oracle_lib, cfg, 2, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs


def test_multi_substep_trajectory(gpu_lib, oracle_lib):
    """1000 substeps of the elastic cube: total mass exact, momentum and kinetic
    energy trajectories within 1e-3 of the FP64 oracle's (sampled every 100)."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=10_000, seed=7)
    mats = [m.derived() for m in cfg["materials"]]
    m = float(mats[0]["particle_mass"])
    state = cfg["state"]
    with Simulation.from_config(cfg) as sim:
        sim.upload(state)
        ref = {k: np.array(v, np.float64) if k != "mat" else v for k, v in state.items()}
        for block in range(10):
            sim.advance(100)
            out = sim.syncDevice()
            ref, g, _ = oracle_lib.substep(ref, cfg["params"], mats, 100, np.float64, want_grids=True)
            p_gpu = m * out["v"].astype(np.float64).sum(0)
            p_ref = m * ref["v"].sum(0)
            ke_gpu = 0.5 * m * (out["v"].astype(np.float64) ** 2).sum()
            ke_ref = 0.5 * m * (ref["v"] ** 2).sum()
            assert abs(g[..., 3].sum() - m * 10_000) < 1e-9 * m * 10_000
            assert np.linalg.norm(p_gpu - p_ref) <= 1e-3 * np.linalg.norm(p_ref) + 1e-9
            assert abs(ke_gpu - ke_ref) <= 1e-3 * ke_ref + 1e-12
        errs = compare_states(out, ref, cfg["params"], ref)
        assert errs["x"] < 1e-5, errs


def test_single_particle_known_answer(gpu_lib):
    """A particle at rest with F = I: after one substep v = dt g and C = 0."""
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    st = {"x": np.array([[0.5, 0.5, 0.5]], np.float32)}
    with Simulation(dt=1e-4, N=16, gravity=-9.8, materials=[M.elastic(1e-5)]) as sim:
        sim.upload(st)
        sim.advance(1)
        out = sim.syncDevice()
    g = np.float32(1e-4) * np.float32(-9.8)
    assert abs(out["v"][0, 1] - g) < 1e-6 * abs(g)
    assert abs(out["v"][0, 0]) < 1e-12 and abs(out["v"][0, 2]) < 1e-12
    assert np.abs(out["C"]).max() < 1e-6


def test_empty_and_outside_particles(gpu_lib, oracle_lib):
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    with Simulation(dt=1e-4, N=16, materials=[M.elastic(1e-5)]) as sim:
        sim.upload({"x": np.zeros((0, 3), np.float32)})
        sim.advance(3)
        sim.sync()
        assert sim.getFullParticleCount() == 0
        # particles fully outside the grid are frozen; one near the upper faces is clipped
        x = np.array([[-0.5, 0.5, 0.5], [0.5, 1.7, 0.5], [0.98, 0.98, 0.98], [0.01, 0.02, 0.5], [0.5, 0.5, 0.5]],
                     np.float32)
        st = {"x": x, "v": np.tile(np.array([[0.1, -0.3, 0.2]], np.float32), (5, 1))}
        sim.upload(st)
        sim.advance(2)
        out = sim.syncDevice()
    full = {"x": x, "v": st["v"], "C": np.zeros((5, 3, 3), np.float32), "F": np.tile(np.eye(3), (5, 1, 1)),
            "Jp": np.ones(5, np.float32), "mat": np.zeros(5, np.uint8)}
    o32, _, _ = oracle_lib.substep(full, {"dt": 1e-4, "N": 16, "gravity": -9.81}, [M.elastic(1e-5).derived()], 2,
                                   np.float32)
    assert np.array_equal(out["x"][:2], x[:2])
    assert np.allclose(out["x"], o32["x"], atol=1e-6)
    assert np.allclose(out["v"], o32["v"], atol=1e-5)


def test_aos_round_trip(gpu_lib):
    from mpm_gb300 import aos, scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.mixed_scene(n=3000, seed=8)
    st = cfg["state"]
    st["C"] = np.random.default_rng(0).standard_normal((3000, 3, 3)).astype(np.float32) * 0.01
    rec = aos.pack(st)
    with Simulation.from_config(cfg) as sim:
        sim.upload_aos(rec)
        back = sim.download_aos()
        soa = sim.download()
    assert np.array_equal(back, rec)
    for k in ("x", "v", "C", "F", "Jp", "mat"):
        assert np.array_equal(soa[k], st[k]), k


def test_check_finite_flags_non_finite_state(gpu_lib):
    """A particle with an infinite velocity (finite position, so every index stays in
    range) spreads inf/NaN through the grid; the kernel records it in the status word
    and mpm_sync reports MPM_ERR_STATE (no trap)."""
    from mpm_gb300 import _lib, scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=2000, seed=9)
    cfg["state"]["v"][7] = [np.inf, 0.0, 0.0]
    with Simulation.from_config(cfg, check_finite=True) as sim:
        sim.upload(cfg["state"])
        sim.advance(3)
        with pytest.raises(_lib.MpmError) as ei:
            sim.sync()
        assert ei.value.code == 3
        sim.sync()  # the status word is cleared once reported
    # non-finite positions are rejected before the context changes
    cfg = scenes.config_elastic(n=2000, seed=9)
    good = {k: v.copy() for k, v in cfg["state"].items()}
    with Simulation.from_config(cfg) as sim:
        sim.upload(good)
        sim.advance(2)
        before = sim.download()
        bad = dict(cfg["state"])
        for row, val in ((3, [np.nan, 0.5, 0.5]), (1999, [0.5, np.inf, 0.5])):
            bad["x"] = good["x"].copy()
            bad["x"][row] = val
            bad["x"] = np.concatenate([bad["x"], good["x"][:100]])  # a larger count as well
            bad = {k: (np.concatenate([good[k], good[k][:100]]) if k != "x" else bad["x"]) for k in good}
            with pytest.raises(_lib.MpmError) as ei:
                sim.upload(bad)
            assert ei.value.code == 1
        # the same count: the upload that puts particles in cell order checks them too
        same = {k: v.copy() for k, v in good.items()}
        same["x"][5] = [0.5, 0.5, np.nan]
        with pytest.raises(_lib.MpmError) as ei:
            sim.upload(same)
        assert ei.value.code == 1
        assert sim.n == len(good["x"]) and sim.substeps == 2
        after = sim.download()
        for k in before:
            assert np.array_equal(before[k], after[k]), k


def test_api_errors(gpu_lib):
    from mpm_gb300 import _lib
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    with pytest.raises(_lib.MpmError):
        Simulation(N=2)
    with Simulation(N=16) as sim:
        with pytest.raises(_lib.MpmError):
            sim.advance(1)  # no materials yet
        sim.set_materials([M.elastic(1e-5)])
        with pytest.raises(_lib.MpmError):
            sim.upload({"x": np.zeros((2, 3), np.float32), "mat": np.array([0, 3], np.uint8)})
        with pytest.raises(_lib.MpmError):
            sim.get_grid(0)  # no completed substep


def _golden_ids():
    from helpers import golden_substep_cases

    return [c[0] for c in golden_substep_cases()]


@pytest.mark.parametrize("case", _golden_ids())
def test_matches_reference_policy_vectors(gpu_lib, case):
    """The CUDA substep against the reference's own policy code run on the host
    (tests/golden/ref_substep.npz, MMSnow elastic / snow / two-material scenes):
    every particle field and the grid after the last P2G within 1e-5 relative."""
    from helpers import golden_substep_cases

    name, cfg, nsteps, expect, grid = next(c for c in golden_substep_cases() if c[0] == case)
    out, (g_p2g, _) = run_gpu(cfg, nsteps, want_grid=True)
    errs = compare_states(out, expect, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs
    assert rel_err(g_p2g, grid) < 1e-5


def test_pinned_host_arrays_take_the_direct_path(gpu_lib):
    """Pinned host arrays are read and written by the conversion kernels over the host link;
    the results equal those of pageable arrays (staged copies), for both layouts, and a
    rejected upload leaves the context unchanged."""
    import ctypes

    import torch

    from mpm_gb300 import _lib, scenes
    from mpm_gb300.simulation import Simulation

    for cfg in (scenes.config_elastic(n=3000, seed=4), scenes.config_liquid(n=5000, seed=4)):
        st = cfg["state"]
        n = len(st["x"])
        liquid = cfg["materials"][0].kind == 3
        keys = ("x", "v", "C", "Jp") if liquid else ("x", "v", "C", "F", "Jp")
        width = {"x": 3, "v": 3, "C": 9, "F": 9, "Jp": 1}
        pin = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(st[k], np.float32).reshape(n, width[k])))
               .pin_memory() for k in keys}
        P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        with Simulation.from_config(cfg) as b:
            b.upload(st)  # staged; sizes the arrays
            staged = b.download()
            _lib.check(b.L.mpm_upload_soa(b.ctx, n, P(pin["x"]), P(pin["v"]), P(pin["C"]), P(pin.get("F")),
                                          P(pin["Jp"]), None), b.ctx)
            direct = b.download()
            for k in staged:
                assert np.array_equal(direct[k], staged[k]), k
            b.advance(20)
            ref = b.download()  # pageable: staged copies
            out = {k: torch.empty((n, width[k]), dtype=torch.float32).pin_memory() for k in keys}
            _lib.check(b.L.mpm_download_soa(b.ctx, P(out["x"]), P(out["v"]), P(out["C"]), P(out.get("F")),
                                            P(out["Jp"]), None), b.ctx)
            for k in keys:
                assert np.array_equal(out[k].numpy().reshape(ref[k].shape), ref[k]), k
            # a non-finite position in pinned arrays: rejected, state kept
            pin["x"][17, 1] = float("nan")
            code = b.L.mpm_upload_soa(b.ctx, n, P(pin["x"]), P(pin["v"]), P(pin["C"]), P(pin.get("F")),
                                      P(pin["Jp"]), None)
            assert code == 1 and b.substeps == 20
            after = b.download()
            for k in ref:
                assert np.array_equal(after[k], ref[k]), k


@pytest.mark.parametrize("liquid", [False, True])
def test_reupload_in_cell_order_matches_a_fresh_upload(gpu_lib, liquid):
    """An upload of the same particle count keeps the device order: each particle goes to the
    slot its id holds (no sort at the next substep). Downloads still return the upload order
    exactly, and the trajectory matches a context that uploaded the same state into new arrays
    and sorted at its first substep (float atomics make the two agree to rounding, not bit for
    bit)."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_liquid(n=6000, seed=9) if liquid else scenes.config_elastic(n=6000, seed=9)
    st = cfg["state"]
    with Simulation.from_config(cfg) as a, Simulation.from_config(cfg) as b:
        a.upload(st)
        a.advance(5)
        a.upload(st)  # same size: the cell-order path
        back = a.download()
        for k in back:
            assert np.array_equal(back[k], np.asarray(st[k], np.float32).reshape(back[k].shape)), k
        b.upload(st)  # new arrays: sorted at the first substep
        a.advance(10)
        b.advance(10)
        ra, rb = a.download(), b.download()
        # natural scales: C of a body nearly at rest is rounding noise around zero
        p = cfg["params"]
        vmax = max(float(np.abs(rb["v"]).max()), abs(p["dt"] * p["gravity"]))
        scale = {"x": 1.0, "v": vmax, "C": 4.0 * p["N"] * vmax, "F": 1.0, "Jp": 1.0}
        for k in scale:
            if k in ra:
                assert np.abs(ra[k] - rb[k]).max() <= 1e-5 * scale[k], k
        if "mat" in ra:
            assert np.array_equal(ra["mat"], rb["mat"])


@pytest.mark.parametrize("shuffled", [False, True])
def test_same_count_upload_keeps_or_restores_cell_order(gpu_lib, shuffled):
    """A same-count upload keeps the device order and counts the slots whose cell key falls
    below their predecessor's. The same scene again keeps the sort schedule (no sort at the
    next substep). The scene's states permuted among the particle indices put the positions
    out of that order: the next substep then sorts first. Either way the download returns the
    upload exactly and the next substep matches a context that uploaded the same state into
    new arrays."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_liquid(n=8000, seed=14)
    st = {k: np.asarray(v).copy() for k, v in cfg["state"].items()}
    perm = np.random.default_rng(15).permutation(len(st["x"]))
    new = {k: v[perm].copy() for k, v in st.items()} if shuffled else st
    with Simulation.from_config(cfg) as a, Simulation.from_config(cfg) as b:
        a.upload(st)
        a.advance(3)
        a.upload(new)
        back = a.download()
        for k in back:
            assert np.array_equal(back[k], np.asarray(new[k], np.float32).reshape(back[k].shape)), k
        l0 = a.launches
        a.advance(1)
        step_launches = a.launches - l0
        # P2G-only, velocity pass, G2P-only; a sort adds its histogram, scan, ranking and gather
        assert step_launches == (7 if shuffled else 3), step_launches
        b.upload(new)
        b.advance(1)
        ra, rb = a.download(), b.download()
        p = cfg["params"]
        vmax = max(float(np.abs(rb["v"]).max()), abs(p["dt"] * p["gravity"]))
        scale = {"x": 1.0, "v": vmax, "C": 4.0 * p["N"] * vmax, "Jp": 1.0}
        for k, sc in scale.items():
            assert np.abs(ra[k] - rb[k]).max() <= 1e-5 * sc, k


def test_upload_loop_ending_without_prefetch_matches_plain_substeps(gpu_lib):
    """Calls that an upload follows end with a G2P-only step (the prefetched P2G would be
    thrown away). When a call then follows without an upload, the skipped P2G is redone:
    the trajectory and the grid readback match a context that never re-uploaded."""
    from mpm_gb300 import scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=5000, seed=12)
    st = cfg["state"]
    with Simulation.from_config(cfg) as a, Simulation.from_config(cfg) as b:
        a.upload(st)
        a.advance(2)
        a.upload(st)  # throws a prefetched P2G away: calls now end with G2P only
        a.advance(1)
        a.upload(st)
        a.advance(1)  # ends with G2P only
        ga = a.get_grid(0)
        a.advance(3)  # no upload in between: the skipped P2G is redone
        b.upload(st)
        b.advance(1)
        gb = b.get_grid(0)
        b.advance(3)
        ra, rb = a.download(), b.download()
        p = cfg["params"]
        vmax = max(float(np.abs(rb["v"]).max()), abs(p["dt"] * p["gravity"]))
        scale = {"x": 1.0, "v": vmax, "C": 4.0 * p["N"] * vmax, "F": 1.0, "Jp": 1.0}
        for k in scale:
            if k in ra:
                assert np.abs(ra[k] - rb[k]).max() <= 1e-5 * scale[k], k
        assert np.abs(ga - gb).max() <= 1e-5 * max(float(np.abs(gb).max()), 1e-6)
        assert a.substeps == b.substeps == 4


def test_argument_validation(gpu_lib, tmp_path):
    """Every entry point rejects bad arguments with its status code (no device work)."""
    import ctypes

    from mpm_gb300 import _lib
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    L = _lib.lib()
    INVALID, IO = 1, 7
    ctx = ctypes.c_void_p()
    for kw in ({"N": 3}, {"N": 1001}, {"dt": 0.0}, {"dt": float("nan")}, {"boundary_mode": 3}):
        p = _lib.MpmParams(float(kw.get("dt", 1e-4)), int(kw.get("N", 16)), -9.8, int(kw.get("boundary_mode", 0)), 3,
                           0, 16, 0)
        assert L.mpm_create(ctypes.byref(p), ctypes.byref(ctx)) == INVALID, kw
    # null contexts and outputs
    assert L.mpm_substep(None, 1) == INVALID
    assert L.mpm_sync(None) == INVALID
    assert L.mpm_surface_mesh(None, 16, 2, None, 0, None) == INVALID
    assert L.mpm_surface_mesh_indexed(None, 16, 2, None, 0, None, 0, None, None) == INVALID
    assert L.mpm_surface_table(None, None) == INVALID
    assert L.mpm_export_particles(None, 0, 0.1, None) == INVALID
    assert L.mpm_render_positions(None, None) == INVALID
    with Simulation(N=16) as sim:
        bad_mats = [(_lib.MpmMaterial * 1)(_lib.MpmMaterial(9, 1e-5, 1000, 1e4, 0.3, 0, 0, 1e30, 0)),
                    (_lib.MpmMaterial * 1)(_lib.MpmMaterial(0, -1.0, 1000, 1e4, 0.3, 0, 0, 1e30, 0))]
        for m in bad_mats:
            assert L.mpm_set_materials(sim.ctx, m, 1) == INVALID
        assert L.mpm_set_materials(sim.ctx, bad_mats[0], 0) == INVALID
        sim.set_materials([M.elastic(1e-5)])
        sim.upload({"x": np.full((100, 3), 0.5, np.float32)})
        p = _lib.MpmParams(1e-4, 32, -9.8, 0, 3, 0, 16, 0)
        assert L.mpm_set_params(sim.ctx, ctypes.byref(p)) == INVALID  # N of a live context
        n = ctypes.c_int64()
        assert L.mpm_export_particles(sim.ctx, 2, 0.1, ctypes.byref(n)) == INVALID
        rec, cnt = ctypes.c_void_p(), ctypes.c_int64()
        assert L.mpm_export_wait(sim.ctx, 1, ctypes.byref(rec), ctypes.byref(cnt)) == INVALID  # nothing exported
        tri = ctypes.c_int64()
        nv = ctypes.c_int64()
        for G, r in ((1, 2), (513, 2), (16, -1), (16, 65)):
            assert L.mpm_surface_mesh(sim.ctx, G, r, None, 0, ctypes.byref(tri)) == INVALID, (G, r)
            assert L.mpm_surface_mesh_indexed(sim.ctx, G, r, None, 0, None, 0, ctypes.byref(nv),
                                              ctypes.byref(tri)) == INVALID, (G, r)
        # a capacity without a buffer is refused; zero capacities only count
        assert L.mpm_surface_mesh_indexed(sim.ctx, 16, 2, None, 4, None, 0, ctypes.byref(nv), ctypes.byref(tri)) == INVALID
        assert L.mpm_surface_mesh_indexed(sim.ctx, 16, 2, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(tri)) == 0
        assert nv.value > 0 and tri.value > 0
        col = (ctypes.c_uint8 * 3)(1, 2, 3)
        img = np.empty(12, np.uint8)
        for w, h, ps in ((0, 10, 2.0), (10, 0, 2.0), (2, 2, 0.0), (2, 2, 100.0)):
            assert L.mpm_render_points(sim.ctx, w, h, ps, col, col, img.ctypes.data_as(ctypes.c_void_p)) == INVALID
        assert L.mpm_write_bgeo(str(tmp_path / "no" / "dir.bgeo").encode(), None, 0) == IO
        # the context still works after all of that
        sim.advance(2)
        sim.sync()
        assert np.isfinite(sim.download(("x",))["x"]).all()
