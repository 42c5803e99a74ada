"""CPU check that the dense float64 torch substep used as the gradient reference
(tests/dense_mpm.py) computes the same substep as the FP64 oracle."""
import numpy as np
import torch

import dense_mpm


def test_dense_matches_oracle_fp64(oracle_lib):
    from mpm_gb300 import scenes

    cfg = scenes.config_differentiable(n=400, seed=3, N=16)
    mats = [m.derived() for m in cfg["materials"]]
    ref, _, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, 5, np.float64)
    st = cfg["state"]
    P = {"dt": float(np.float32(cfg["params"]["dt"])), "N": 16, "vol": float(mats[0]["particle_volume"]),
         "mass": float(mats[0]["particle_mass"]), "gravity": float(np.float32(cfg["params"]["gravity"]))}
    t = lambda a: torch.tensor(np.asarray(a, np.float64))  # noqa: E731
    x, v, C, F, J = t(st["x"]), t(st["v"]), t(st["C"]), t(st["F"]), t(st["Jp"])
    mu, lam = float(mats[0]["mu0"]), float(mats[0]["lambda0"])
    for _ in range(5):
        x, v, C, F = dense_mpm.substep(x, v, C, F, J, mu, lam, P)
    assert np.abs(x.numpy() - ref["x"]).max() < 1e-12
    assert np.abs(v.numpy() - ref["v"]).max() < 1e-9 * max(1.0, np.abs(ref["v"]).max())
    assert np.abs(C.numpy() - ref["C"]).max() < 1e-8 * max(1.0, np.abs(ref["C"]).max())
    assert np.abs(F.numpy() - ref["F"]).max() < 1e-11


def test_dense_gradient_finite_difference():
    """The dense reference's autograd gradient agrees with its own central differences."""
    from mpm_gb300 import scenes

    cfg = scenes.config_differentiable(n=200, seed=4, N=16)
    st = cfg["state"]
    m = cfg["materials"][0]
    P = {"dt": 1e-4, "N": 16, "vol": m.particle_volume, "mass": m.density * m.particle_volume, "gravity": -9.8}
    t = lambda a: torch.tensor(np.asarray(a, np.float64))  # noqa: E731
    target = torch.tensor([0.6, 0.3, 0.5], dtype=torch.float64)

    def loss(v0, E):
        x, _, _, _ = dense_mpm.rollout(t(st["x"]), v0, t(st["C"]), t(st["F"]), t(st["Jp"]), E, 0.3, P, 4)
        return ((x.mean(0) - target) ** 2).sum()

    v0 = t(st["v"]).requires_grad_(True)
    E = torch.tensor(1e4, dtype=torch.float64, requires_grad=True)
    L = loss(v0, E)
    gv, gE = torch.autograd.grad(L, (v0, E))
    u = torch.randn_like(v0, generator=torch.Generator().manual_seed(0))
    eps = 1e-6
    fd = (loss(v0.detach() + eps * u, E.detach()) - loss(v0.detach() - eps * u, E.detach())) / (2 * eps)
    assert abs(fd - (gv * u).sum()) < 1e-5 * abs(fd) + 1e-14
    fdE = (loss(v0.detach(), E.detach() * (1 + 1e-6)) - loss(v0.detach(), E.detach() * (1 - 1e-6))) / (2e-6 * 1e4)
    assert abs(fdE - gE) < 1e-4 * abs(fdE) + 1e-16
