"""GPU tests of the snow adjoint: MMSnow's plasticity (the SVD, the singular-value clamp
and the Jp update of endOfStepMutation, include/MaterialModel.cuh:95-115) and its
hardening-scaled stress (computePF, :85-93) differentiated by hand (mpm_gb300/csrc/
adjoint.cu), against central finite differences of the FP64 oracle.  Bar: 1e-3 relative.

The clamp has no derivative at the band's edges, so each scene keeps every particle
clearly on one side of them, and the test checks that on every substep with the FP64
oracle: the singular values of F^ = (I + dt C') F stay at least 1e-3 away from
[0.975, 1.0075] (the finite-difference steps move them by less than 1e-6):
  * inside: F starts at random stretches with singular values in [0.985, 0.998] and Jp in
    [0.95, 1.05], small velocities; 12 substeps, the clamp inactive;
  * outside: F starts at 0.97 I under a compression of 40/s, so every singular value is
    clamped to 0.975 on every substep and Jp drops from 1 to 0.93 (6 substeps): the clamp's
    zero derivative, the Jp update and the hardening exp(10 (1 - Jp)) all act.
Losses: L = ||COM(x_final) - (0.6, 0.3, 0.5)||^2 for the velocity directions, and the
spread L2 = mean ||x_final - COM||^2 for the elastic constants.  The constants are checked
as the adjoint reports them, dL2/dmu0 and dL2/dlambda0, against differences of mu0 and
lambda0 by steps exactly representable in float32 (the reference derives mu0 and lambda0 in
float, so steps of E or nu are rounded there); these converge to 1e-9 over steps of 1e-4 to
1e-2.  dL/dE and dL/dnu follow from them by the exact chain rule of autograd.lame_grad."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TARGET = np.array([0.6, 0.3, 0.5])


def rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def snow_case(kind, n=3000, seed=11, N=24):
    from mpm_gb300 import materials as M
    from mpm_gb300 import scenes

    rng = np.random.default_rng(seed)
    c = np.array([0.5, 0.5, 0.5])
    r = 0.08
    x = scenes.sample_sphere(rng, n, c, r).astype(np.float64)
    st = scenes._empty_state(n)
    st["x"] = x.astype(np.float32)
    if kind == "inside":
        R = rotations(rng, n)
        s = rng.uniform(0.985, 0.998, (n, 3))
        st["F"] = np.einsum("nij,nj,nkj->nik", R, s, R).astype(np.float32)
        st["Jp"] = rng.uniform(0.95, 1.05, n).astype(np.float32)
        st["v"] = (0.02 * rng.standard_normal((n, 3)) + np.cross([0.0, 0.0, 1.0], x - c)).astype(np.float32)
    else:
        st["F"] = np.tile(0.97 * np.eye(3), (n, 1, 1)).astype(np.float32)
        st["v"] = (-40.0 * (x - c) + 0.01 * rng.standard_normal((n, 3))).astype(np.float32)
    params = {"dt": 1e-4, "N": N, "gravity": -9.8, "boundary_mode": 0, "boundary_cells": 3}
    return {"state": st, "params": params, "materials": [M.snow(4.0 / 3.0 * np.pi * r ** 3 / n)]}


def clamp_margin(oracle_lib, cfg, nsteps):
    """Smallest distance of a singular value of F^ to the clamp band's edges over all
    particles and substeps (FP64 oracle, one substep at a time); also the Jp range."""
    mat = cfg["materials"][0].derived()
    lo, hi = float(np.float32(mat["clamp_lo"])), float(np.float32(mat["clamp_hi"]))
    st = {k: np.array(v, np.float64) if k != "mat" else v for k, v in cfg["state"].items()}
    worst, jlo, jhi = np.inf, np.inf, -np.inf
    for _ in range(nsteps):
        nxt, _, _ = oracle_lib.substep(st, cfg["params"], [mat], 1, np.float64)
        Fh = np.einsum("nij,njk->nik", np.eye(3) + cfg["params"]["dt"] * nxt["C"], st["F"])
        s = np.linalg.svd(Fh, compute_uv=False)
        worst = min(worst, float(np.minimum(np.abs(s - lo), np.abs(s - hi)).min()))
        jlo, jhi = min(jlo, float(nxt["Jp"].min())), max(jhi, float(nxt["Jp"].max()))
        st = nxt
    return worst, jlo, jhi


def losses(x):
    x = x.astype(np.float64)
    c = x.mean(0)
    return float(((c - TARGET) ** 2).sum()), float(((x - c) ** 2).sum(1).mean())


@pytest.mark.parametrize("kind,nsteps,ckpt", [("inside", 12, 4), ("outside", 6, 3)])
def test_snow_adjoint_matches_fp64_finite_differences(gpu_lib, oracle_lib, kind, nsteps, ckpt):
    from mpm_gb300.autograd import DiffSim, lame_grad

    cfg = snow_case(kind)
    st = cfg["state"]
    n = st["x"].shape[0]
    m = cfg["materials"][0]
    margin, jlo, jhi = clamp_margin(oracle_lib, cfg, nsteps)
    assert margin > 1e-3, margin
    if kind == "outside":
        assert jhi < 0.98 and jlo > 0.9, (jlo, jhi)  # the plastic volume change acts

    sim = DiffSim(cfg["params"], m, n, nsteps, ckpt)
    xo, _ = sim.forward(st, nsteps)
    x64 = xo.astype(np.float64)
    com = x64.mean(0)
    g_com = sim.backward(np.tile(2.0 * (com - TARGET) / n, (n, 1)))
    g_spr = sim.backward(2.0 * (x64 - com) / n)
    sim.close()
    base = m.derived()

    def run(v0=None, **consts):
        d = dict(base)
        d.update(consts)
        s = dict(st)
        if v0 is not None:
            s["v"] = v0
        out, _, _ = oracle_lib.substep(s, cfg["params"], [d], nsteps, np.float64)
        return losses(out["x"])

    rng = np.random.default_rng(3)
    v0 = st["v"].astype(np.float64)
    for u in (np.array([1.0, -0.5, 0.25]) + 0.2 * rng.standard_normal(v0.shape), rng.standard_normal(v0.shape)):
        eps = 1e-4
        fd = (run(v0=v0 + eps * u)[0] - run(v0=v0 - eps * u)[0]) / (2 * eps)
        ad = float((g_com["v"].astype(np.float64) * u).sum())
        assert abs(ad - fd) < 1e-3 * abs(fd), (kind, ad, fd)
    for name in ("mu0", "lambda0"):
        val = np.float32(base[name])
        hp, hm = float(np.float32(val * 1.001)), float(np.float32(val * 0.999))
        fd = (run(**{name: hp})[1] - run(**{name: hm})[1]) / (hp - hm)
        assert abs(g_spr[name] - fd) < 1e-3 * abs(fd), (kind, name, g_spr[name], fd)
    gE, gnu = lame_grad(m.E, m.nu, g_spr["mu0"], g_spr["lambda0"])
    assert np.isfinite(gE) and np.isfinite(gnu)
