"""GPU tests of the hand-written adjoint (mpm_diff_*): gradients of
L = ||COM(x_final) - target||^2 w.r.t. the initial velocities and positions and E, nu,
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


def loss_grad_x(x):
    com = x.astype(np.float64).mean(0)
    return np.tile(2.0 * (com - TARGET) / x.shape[0], (x.shape[0], 1)), float(((com - TARGET) ** 2).sum())


def gpu_grads(cfg, nsteps, ckpt):
    from mpm_gb300.autograd import DiffSim, lame_grad

    m = cfg["materials"][0]
    sim = DiffSim(cfg["params"], m, cfg["state"]["x"].shape[0], nsteps, ckpt)
    xo, _ = sim.forward(cfg["state"], nsteps)
    gx, L = loss_grad_x(xo)
    g = sim.backward(gx)
    g["E"], g["nu"] = lame_grad(m.E, m.nu, g["mu0"], g["lambda0"])
    sim.close()
    return g, L


def dense_grads(cfg, nsteps):
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
    assert abs(g["E"] - r["E"]) < 1e-3 * abs(r["E"]) + 1e-12, (g["E"], r["E"])
    assert abs(g["nu"] - r["nu"]) < 1e-3 * abs(r["nu"]) + 1e-12, (g["nu"], r["nu"])


def test_adjoint_matches_fp64_finite_differences(gpu_lib, oracle_lib):
    """Directional derivatives along random velocity perturbations, and dL/dE, dL/dnu,
    against central differences of the FP64 oracle."""
    cfg = small_case(n=2000, seed=6)
    nsteps = 12
    g, _ = gpu_grads(cfg, nsteps, 4)
    st = cfg["state"]
    m = cfg["materials"][0]

    def L_of(v0=None, E=None, nu=None):
        from mpm_gb300 import materials as M

        mm = M.fixed_corotated(m.particle_volume, m.density, E if E is not None else m.E, nu if nu is not None else m.nu)
        s = dict(st)
        if v0 is not None:
            s["v"] = v0
        out, _, _ = oracle_lib.substep(s, cfg["params"], [mm.derived()], nsteps, np.float64)
        com = out["x"].mean(0)
        return float(((com - TARGET) ** 2).sum())

    rng = np.random.default_rng(0)
    v0 = st["v"].astype(np.float64)
    for _ in range(3):
        u = rng.standard_normal(v0.shape)
        eps = 1e-3
        fd = (L_of(v0=v0 + eps * u) - L_of(v0=v0 - eps * u)) / (2 * eps)
        ad = float((g["v"].astype(np.float64) * u).sum())
        assert abs(ad - fd) < 1e-3 * abs(fd) + 1e-12, (ad, fd)
    for name, val in (("E", m.E), ("nu", m.nu)):
        h = 1e-3 * val
        fd = (L_of(**{name: val + h}) - L_of(**{name: val - h})) / (2 * h)
        assert abs(g[name] - fd) < 1e-3 * abs(fd) + 1e-12, (name, g[name], fd)


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


def test_full_size_differentiable_config(gpu_lib):
    """100k particles, N=64, 256 substeps, checkpoint every 16: the gradient is finite
    and its directional derivative matches the GPU forward's central difference."""
    from mpm_gb300 import scenes
    from mpm_gb300.autograd import DiffSim

    cfg = scenes.config_differentiable()
    st = cfg["state"]
    n = st["x"].shape[0]
    sim = DiffSim(cfg["params"], cfg["materials"][0], n, 256, 16)
    xo, _ = sim.forward(st, 256)
    gx, L = loss_grad_x(xo)
    g = sim.backward(gx)
    assert np.isfinite(g["v"]).all() and np.isfinite(g["x"]).all()
    rng = np.random.default_rng(1)
    # a common drift plus noise: the loss sees the centre of mass, so the common part
    # gives a finite difference well above FP32 rounding
    u = (np.array([1.0, 0.5, -0.3]) + 0.1 * rng.standard_normal(st["v"].shape)).astype(np.float32)
    eps = 2e-2

    def L_of(v):
        s = dict(st)
        s["v"] = v
        x, _ = sim.forward(s, 256)
        return loss_grad_x(x)[1]

    fd = (L_of(st["v"] + eps * u) - L_of(st["v"] - eps * u)) / (2 * eps)
    ad = float((g["v"].astype(np.float64) * u).sum())
    assert abs(ad - fd) < 2e-2 * abs(fd), (ad, fd)
    sim.close()
