"""A small dense re-implementation of the substep in float64 torch, for gradient checks.

Test infrastructure only: it restates the reference substep (src/mpm.cu:14-178 with
MMFixedCorotated, include/MaterialModel.cuh:56-61) with differentiable torch ops, so
autograd gives a reference gradient for the hand-written adjoint kernels.  The polar
rotation uses the Newton iteration R <- (R + R^-T) / 2, which is differentiable at
F = I where an SVD's gradient is not.  Boundary rule: the reference's 0.05 fraction.
"""
import itertools

import torch

OFFSETS = list(itertools.product(range(3), range(3), range(3)))


def polar_rotation(F, iters=12):
    R = F
    for _ in range(iters):
        R = 0.5 * (R + torch.linalg.inv(R).transpose(-1, -2))
    return R


def substep(x, v, C, F, Jp, mu, lam, P):
    """One substep; P: dict with dt, N, vol, mass, gravity (floats/ints)."""
    dt, N = P["dt"], P["N"]
    dx = 1.0 / N
    dxi = float(N)
    dinv = 4.0 * dxi * dxi
    m = P["mass"]
    xg = x * dxi
    base = (xg - 0.5).detach().to(torch.int64)
    fx = xg - base.to(x.dtype)
    w = torch.stack([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2], dim=-1)
    R = polar_rotation(F)
    eye = torch.eye(3, dtype=x.dtype)
    PF = 2.0 * mu * (F - R) @ F.transpose(-1, -2) + (lam * (Jp - 1.0) * Jp)[:, None, None] * eye
    s = -dinv * dt * P["vol"]
    A = s * PF + m * C
    cells = N * N * N
    mv = torch.zeros(cells, 3, dtype=x.dtype)
    mg = torch.zeros(cells, dtype=x.dtype)
    nodes = []
    for a, b, c in OFFSETS:
        off = torch.tensor([a, b, c])
        node = base + off
        dpos = node.to(x.dtype) * dx - x
        wt = w[:, 0, a] * w[:, 1, b] * w[:, 2, c]
        idx = (node[:, 0] * N + node[:, 1]) * N + node[:, 2]
        contrib = m * v + (A @ dpos[:, :, None])[:, :, 0]
        mv = mv.index_add(0, idx, wt[:, None] * contrib)
        mg = mg.index_add(0, idx, wt * m)
        nodes.append((idx, wt, dpos))
    # grid op (src/mpm.cu:76-107)
    has = mg > 0
    vg = torch.where(has[:, None], mv / torch.where(has, mg, torch.ones_like(mg))[:, None], mv)
    grav = torch.zeros(cells, 3, dtype=x.dtype)
    grav[:, 1] = dt * P["gravity"]
    vg = vg + torch.where(has[:, None], grav, torch.zeros_like(grav))
    ii = torch.arange(cells)
    gi, gj, gk = ii // (N * N), (ii // N) % N, ii % N
    b_ = 0.05
    xs, ys, zs = gi.to(x.dtype) / N, gj.to(x.dtype) / N, gk.to(x.dtype) / N
    sticky = has & ((xs < b_) | (xs > 1 - b_) | (ys > 1 - b_) | (zs < b_) | (zs > 1 - b_))
    floor = has & (ys < b_)
    vg = torch.where(sticky[:, None], torch.zeros_like(vg), vg)
    vy = torch.where(floor, torch.clamp(vg[:, 1], min=0.0), vg[:, 1])
    vg = torch.stack([vg[:, 0], vy, vg[:, 2]], dim=1)
    # G2P
    v1 = torch.zeros_like(v)
    C1 = torch.zeros_like(C)
    for idx, wt, dpos in nodes:
        vi = vg[idx]
        v1 = v1 + wt[:, None] * vi
        C1 = C1 + dinv * wt[:, None, None] * vi[:, :, None] * dpos[:, None, :]
    F1 = (eye + dt * C1) @ F
    x1 = x + dt * v1
    return x1, v1, C1, F1


def rollout(x, v, C, F, Jp, E, nu, P, nsteps):
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    for _ in range(nsteps):
        x, v, C, F = substep(x, v, C, F, Jp, mu, lam, P)
    return x, v, C, F
