"""GPU tests of the hand-written adjoint (mpm_diff_*): gradients w.r.t. the initial
velocities and positions and E, nu of two losses of the final positions,
  L  = ||COM(x_final) - target||^2   (the differentiable workload's loss), and
  L2 = mean ||x_final - COM||^2      (the spread, which depends on E and nu: the COM of a
                                      body clear of the walls does not, since P2G and G2P
                                      conserve momentum, so dL/dE = dL/dnu = 0),
against (1) autograd through the dense float64 torch substep (tests/dense_mpm.py) and
(2) central finite differences of the FP64 CPU oracle.  Bar: 1e-3 relative."""
import numpy as np
import pytest
import torch

import dense_mpm

pytestmark = pytest.mark.gpu

TARGET = np.array([0.6, 0.3, 0.5])


def small_case(n=300, seed=5, N=16):
    from mpm_gb300 import scenes

    cfg = scenes.config_differentiable(n=n, seed=seed, N=N)
    return cfg


def loss_grad_x(x, loss="com"):
    """dL/dx_final and L for the COM loss or the spread."""
    x = x.astype(np.float64)
    com = x.mean(0)
    if loss == "spread":
        return 2.0 * (x - com) / x.shape[0], float(((x - com) ** 2).sum(1).mean())
    return np.tile(2.0 * (com - TARGET) / x.shape[0], (x.shape[0], 1)), float(((com - TARGET) ** 2).sum())


def sheared_case(n=300, seed=5, N=16):
    """The small case with a coherent initial velocity (a shear plus a compression of the
    body, ~10/s): strains reach ~5e-2 within 48 substeps, so the elastic constants move the
    spread far above FP32 rounding."""
    cfg = small_case(n, seed, N)
    x = cfg["state"]["x"].astype(np.float64)
    G = 5.0 * np.array([[-1.0, 2.0, 0.0], [0.5, -1.5, 0.0], [0.0, 1.0, -2.0]])
    cfg["state"]["v"] = (cfg["state"]["v"] + (x - x.mean(0)) @ G.T).astype(np.float32)
    return cfg


def gpu_grads(cfg, nsteps, ckpt, loss="com"):
    from mpm_gb300.autograd import DiffSim, lame_grad

    m = cfg["materials"][0]
    sim = DiffSim(cfg["params"], m, cfg["state"]["x"].shape[0], nsteps, ckpt)
    xo, _ = sim.forward(cfg["state"], nsteps)
    gx, L = loss_grad_x(xo, loss)
    g = sim.backward(gx)
    g["E"], g["nu"] = lame_grad(m.E, m.nu, g["mu0"], g["lambda0"])
    sim.close()
    return g, L


def dense_grads(cfg, nsteps, loss="com"):
    st = cfg["state"]
    m = cfg["materials"][0]
    d = m.derived()
    P = {"dt": float(np.float32(cfg["params"]["dt"])), "N": cfg["params"]["N"], "vol": float(d["particle_volume"]),
         "mass": float(d["particle_mass"]), "gravity": float(np.float32(cfg["params"]["gravity"]))}
    t = lambda a: torch.tensor(np.asarray(a, np.float64))  # noqa: E731
    x0 = t(st["x"]).requires_grad_(True)
    v0 = t(st["v"]).requires_grad_(True)
    E = torch.tensor(float(m.E), dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(float(m.nu), dtype=torch.float64, requires_grad=True)
    x, _, _, _ = dense_mpm.rollout(x0, v0, t(st["C"]), t(st["F"]), t(st["Jp"]), E, nu, P, nsteps)
    if loss == "spread":
        L = ((x - x.mean(0)) ** 2).sum(1).mean()
    else:
        L = ((x.mean(0) - torch.tensor(TARGET)) ** 2).sum()
    gx, gv, gE, gnu = torch.autograd.grad(L, (x0, v0, E, nu))
    return {"x": gx.numpy(), "v": gv.numpy(), "E": float(gE), "nu": float(gnu)}, float(L)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("nsteps,ckpt", [(1, 1), (8, 3), (16, 16)])
def test_adjoint_matches_dense_autograd(gpu_lib, nsteps, ckpt):
    cfg = small_case()
    g, L = gpu_grads(cfg, nsteps, ckpt)
    r, Lr = dense_grads(cfg, nsteps)
    assert abs(L - Lr) < 1e-5 * Lr
    assert rel(g["v"], r["v"]) < 1e-3, rel(g["v"], r["v"])
    assert rel(g["x"], r["x"]) < 1e-3, rel(g["x"], r["x"])
    # the COM loss does not depend on E or nu: both sides vanish
    assert abs(g["E"]) < 1e-9 * abs(Lr) and abs(r["E"]) < 1e-9 * abs(Lr), (g["E"], r["E"])


@pytest.mark.parametrize("nsteps,ckpt", [(24, 8), (48, 16)])
def test_elastic_constant_gradients_match_dense_autograd(gpu_lib, nsteps, ckpt):
    """dL2/dE and dL2/dnu of the spread of a sheared body, and its dL2/dx0, dL2/dv0, against
    autograd through the dense float64 substep; the gradients are far from zero."""
    cfg = sheared_case()
    g, L = gpu_grads(cfg, nsteps, ckpt, "spread")
    r, Lr = dense_grads(cfg, nsteps, "spread")
    assert abs(L - Lr) < 1e-5 * Lr
    m = cfg["materials"][0]
    # the constants matter: E's whole value moves the spread by more than 1e-6 of itself
    # (FP32 rounding of the positions moves it by ~1e-9)
    assert abs(r["E"]) * m.E > 1e-6 * Lr, (r["E"], Lr)
    assert abs(g["E"] - r["E"]) < 1e-3 * abs(r["E"]), (g["E"], r["E"])
    assert abs(g["nu"] - r["nu"]) < 1e-3 * abs(r["nu"]), (g["nu"], r["nu"])
    assert rel(g["v"], r["v"]) < 1e-3, rel(g["v"], r["v"])
    assert rel(g["x"], r["x"]) < 1e-3, rel(g["x"], r["x"])


def test_adjoint_matches_fp64_finite_differences(gpu_lib, oracle_lib):
    """Directional derivatives of the COM loss along random velocity perturbations, and
    dL2/dmu0, dL2/dlambda0 of the spread of a sheared body, against central differences of
    the FP64 oracle (steps of mu0 and lambda0 exactly representable in float32)."""
    cfg = small_case(n=2000, seed=6)
    nsteps = 12
    g, _ = gpu_grads(cfg, nsteps, 4)
    st = cfg["state"]
    m = cfg["materials"][0]

    base = m.derived()

    def L_of(v0=None, state=None, loss="com", nsteps=nsteps, **consts):
        d = dict(base)
        d.update(consts)
        s = dict(state if state is not None else st)
        if v0 is not None:
            s["v"] = v0
        out, _, _ = oracle_lib.substep(s, cfg["params"], [d], nsteps, np.float64)
        return loss_grad_x(out["x"], loss)[1]

    rng = np.random.default_rng(0)
    v0 = st["v"].astype(np.float64)
    for _ in range(3):
        u = rng.standard_normal(v0.shape)
        eps = 1e-3
        fd = (L_of(v0=v0 + eps * u) - L_of(v0=v0 - eps * u)) / (2 * eps)
        ad = float((g["v"].astype(np.float64) * u).sum())
        assert abs(ad - fd) < 1e-3 * abs(fd) + 1e-12, (ad, fd)
    sh = sheared_case(n=2000, seed=6)
    g2, _ = gpu_grads(sh, 48, 16, "spread")
    for name in ("mu0", "lambda0"):
        val = np.float32(base[name])
        hp, hm = float(np.float32(val * 1.001)), float(np.float32(val * 0.999))
        fd = (L_of(state=sh["state"], loss="spread", nsteps=48, **{name: hp}) -
              L_of(state=sh["state"], loss="spread", nsteps=48, **{name: hm})) / (hp - hm)
        if name == "lambda0":
            # the stress's lambda term is lambda0 (Jp - 1) Jp with the stored Jp, which stays 1
            # for this material (the reference's stress uses Jp, not det F): no dependence
            assert fd == 0.0 and g2[name] == 0.0, (g2[name], fd)
            continue
        assert abs(g2[name] - fd) < 1e-3 * abs(fd), (name, g2[name], fd)


def test_autograd_function(gpu_lib):
    from mpm_gb300.autograd import DiffSim, rollout

    cfg = small_case(n=500, seed=7)
    st = cfg["state"]
    m = cfg["materials"][0]
    sim = DiffSim(cfg["params"], m, 500, 10, 5)
    x0 = torch.tensor(st["x"], requires_grad=True)
    v0 = torch.tensor(st["v"], requires_grad=True)
    E = torch.tensor(m.E, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(m.nu, dtype=torch.float64, requires_grad=True)
    x = rollout(x0, v0, E, nu, sim, 10)
    L = ((x.double().mean(0) - torch.tensor(TARGET)) ** 2).sum()
    L.backward()
    r, _ = dense_grads(cfg, 10)
    assert rel(v0.grad.numpy(), r["v"]) < 1e-3
    assert abs(E.grad.item() - r["E"]) < 1e-3 * abs(r["E"]) + 1e-12
    sim.close()


def test_full_size_differentiable_config(gpu_lib, oracle_lib):
    """The differentiable workload in full: 100,000 fixed-corotated particles, N = 64, 256
    substeps, a checkpoint every 16.  The GPU adjoint (FP32 forward, hand-written adjoint
    kernels) against central differences of the FP64 oracle, bar 1e-3 relative:
      * dL/dv0 of the workload's loss L = ||COM(x_final) - (0.6, 0.3, 0.5)||^2 along two
        seeded directions (a common drift plus noise, and pure noise);
      * dL2/dmu0 and dL2/dlambda0 of the spread L2 = mean ||x_final - COM||^2, against
        differences of mu0 and lambda0 by steps exactly representable in float32 (the
        reference derives them in float, so steps of E or nu would be rounded there); dL/dE
        and dL/dnu follow by the exact chain rule of lame_grad.  The COM loss does
        not depend on E or nu while the body flies clear of the walls (P2G and G2P conserve
        momentum, so the COM follows the initial mean velocity and gravity): its dL/dE and
        dL/dnu vanish up to rounding.  Both the adjoint's and the finite difference's are
        checked to be negligible: relative to L, below 1e-3 of the spread's relative
        sensitivity (dL2/dmu0) / L2."""
    from mpm_gb300 import materials as M
    from mpm_gb300 import scenes
    from mpm_gb300.autograd import DiffSim, lame_grad

    cfg = scenes.config_differentiable()
    st = cfg["state"]
    n = st["x"].shape[0]
    nsteps = 256
    assert n == 100_000 and cfg["params"]["N"] == 64 and cfg["checkpoint_every"] == 16
    m = cfg["materials"][0]
    sim = DiffSim(cfg["params"], m, n, nsteps, 16)
    xo, _ = sim.forward(st, nsteps)
    gx, L = loss_grad_x(xo)
    g = sim.backward(gx)
    assert np.isfinite(g["v"]).all() and np.isfinite(g["x"]).all()
    gE, gnu = lame_grad(m.E, m.nu, g["mu0"], g["lambda0"])
    x64 = xo.astype(np.float64)
    com = x64.mean(0)
    g2 = sim.backward(2.0 * (x64 - com) / n)
    g2E, g2nu = lame_grad(m.E, m.nu, g2["mu0"], g2["lambda0"])
    sim.close()

    base = m.derived()

    def run(v0=None, **consts):
        d = dict(base)
        d.update(consts)
        s = dict(st)
        if v0 is not None:
            s["v"] = v0
        out, _, _ = oracle_lib.substep(s, cfg["params"], [d], nsteps, np.float64)
        x = out["x"]
        c = x.mean(0)
        return float(((c - TARGET) ** 2).sum()), float(((x - c) ** 2).sum(1).mean())

    rng = np.random.default_rng(1)
    v0 = st["v"].astype(np.float64)
    dirs = [np.array([1.0, 0.5, -0.3]) + 0.1 * rng.standard_normal(v0.shape), rng.standard_normal(v0.shape)]
    for u in dirs:
        eps = 1e-3
        fd = (run(v0=v0 + eps * u)[0] - run(v0=v0 - eps * u)[0]) / (2 * eps)
        ad = float((g["v"].astype(np.float64) * u).sum())
        assert abs(ad - fd) < 1e-3 * abs(fd), (ad, fd)
    L2 = float(((x64 - com) ** 2).sum(1).mean())
    for name in ("mu0", "lambda0"):
        val = np.float32(base[name])
        hp, hm = float(np.float32(val * 1.001)), float(np.float32(val * 0.999))
        lp, lm = run(**{name: hp}), run(**{name: hm})
        fd2 = (lp[1] - lm[1]) / (hp - hm)
        fd1 = (lp[0] - lm[0]) / (hp - hm)
        print(f"{name}: spread adjoint {g2[name]:.6e} fd {fd2:.6e}; COM adjoint {g[name]:.3e} fd {fd1:.3e}")
        if name == "lambda0":
            # lambda0 (Jp - 1) Jp with Jp = 1 throughout: the spread does not depend on lambda0
            assert fd2 == 0.0 and g2[name] == 0.0 and fd1 == 0.0 and g[name] == 0.0, (g2[name], fd2)
            continue
        assert abs(g2[name] - fd2) < 1e-3 * abs(fd2), (name, g2[name], fd2)
        negligible = 1e-3 * abs(fd2) / L2 * L
        assert abs(fd1) < negligible and abs(g[name]) < negligible, (name, g[name], fd1, negligible)
    assert np.isfinite([gE, gnu, g2E, g2nu]).all()


def test_frozen_particles_pass_the_adjoint_through(gpu_lib):
    """Particles completely outside the domain are frozen in the forward (no G2P, no P2G),
    so their adjoint passes through every substep unchanged and they touch nobody else's.
    With a linear loss r . x_final on 20 such particles added to the sheared body (spread
    loss), over 8 substeps in segments of 3, 3 and 2 (every kernel of the backward, both
    segment ends included): their dL/dx0 is exactly r and their dL/dv0 exactly 0, and the
    body's gradients equal those of the body alone to rounding (the extra particles change
    the cell order, so the P2G sums round differently)."""
    base = sheared_case()
    g0, _ = gpu_grads(base, 8, 3, "spread")
    n0 = base["state"]["x"].shape[0]
    rng = np.random.default_rng(11)
    k = 20
    extra = {"x": rng.uniform(1.3, 1.9, (k, 3)), "v": rng.standard_normal((k, 3)),
             "C": 0.1 * rng.standard_normal((k, 3, 3)), "F": np.tile(np.eye(3), (k, 1, 1)), "Jp": np.ones(k)}
    cfg = sheared_case()
    for f, a in extra.items():
        cfg["state"][f] = np.concatenate([cfg["state"][f], a.astype(np.float32)])
    from mpm_gb300.autograd import DiffSim

    m = cfg["materials"][0]
    sim = DiffSim(cfg["params"], m, n0 + k, 8, 3)
    xo, _ = sim.forward(cfg["state"], 8)
    assert np.array_equal(xo[n0:], cfg["state"]["x"][n0:])  # frozen in the forward
    gx, _ = loss_grad_x(xo[:n0], "spread")
    r = rng.standard_normal((k, 3)).astype(np.float32)
    g = sim.backward(np.concatenate([gx, r]))
    sim.close()
    assert np.array_equal(g["x"][n0:], r)
    assert not g["v"][n0:].any()
    assert rel(g["x"][:n0], g0["x"]) < 1e-4, rel(g["x"][:n0], g0["x"])
    assert rel(g["v"][:n0], g0["v"]) < 1e-4, rel(g["v"][:n0], g0["v"])
    assert abs(g["mu0"] - g0["mu0"]) < 1e-4 * abs(g0["mu0"]), (g["mu0"], g0["mu0"])
