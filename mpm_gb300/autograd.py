"""Differentiable MLS-MPM substeps for PyTorch.

:class:`DiffSim` wraps the checkpointed forward / adjoint C ABI (mpm_diff_* in
include/mpm_gb300.h); :class:`MPMRollout` is the torch.autograd.Function that a
training loop calls: it maps the initial particle velocities, positions and the
material's E and nu to the final positions, and its backward pass runs the
hand-written adjoint kernels on the GPU.  Gradients w.r.t. E and nu come from the
adjoint's dL/dmu0 and dL/dlambda0 through the Lame relations the reference uses
(include/MaterialModel.cuh:50-54).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .materials import FIXED_COROTATED, SNOW, Material


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a, shape):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shape))


class DiffSim:
    def __init__(self, params: dict, material: Material, n: int, max_steps: int, checkpoint_every: int = 16):
        if material.kind not in (FIXED_COROTATED, SNOW):
            raise ValueError("the adjoint covers the fixed-corotated and snow materials")
        self.L = _lib.lib()
        self.params = _lib.MpmParams(float(params["dt"]), int(params["N"]), float(params.get("gravity", -9.81)),
                                     int(params.get("boundary_mode", 0)), int(params.get("boundary_cells", 3)), 0, 0, 0)
        self.material = material
        h = ctypes.c_void_p()
        code = self.L.mpm_diff_create(ctypes.byref(self.params), ctypes.byref(self._mat(material)), int(n),
                                      int(max_steps), int(checkpoint_every), ctypes.byref(h))
        if code != 0:
            raise _lib.MpmError(code, "mpm_diff_create failed")
        self.h = h
        self.n = int(n)

    @staticmethod
    def _mat(m: Material):
        return _lib.MpmMaterial(int(m.kind), float(m.particle_volume), float(m.density), float(m.E), float(m.nu),
                                float(m.hardening), float(m.clamp_lo), float(m.clamp_hi), float(m.bulk))

    def set_E_nu(self, E: float, nu: float):
        self.material.E = float(E)
        self.material.nu = float(nu)
        _lib.check(self.L.mpm_diff_set_material(self.h, ctypes.byref(self._mat(self.material))))

    def forward(self, state: dict, nsteps: int):
        n = self.n
        x = _f32(state["x"], (n, 3))
        v = _f32(state.get("v", np.zeros((n, 3))), (n, 3))
        C = _f32(state.get("C", np.zeros((n, 3, 3))), (n, 9))
        F = _f32(state.get("F", np.tile(np.eye(3), (n, 1, 1))), (n, 9))
        J = _f32(state.get("Jp", np.ones(n)), (n,))
        xo = np.empty((n, 3), np.float32)
        vo = np.empty((n, 3), np.float32)
        _lib.check(self.L.mpm_diff_forward(self.h, _ptr(x), _ptr(v), _ptr(C), _ptr(F), _ptr(J), int(nsteps), _ptr(xo),
                                           _ptr(vo)))
        return xo, vo

    def backward(self, gx_final, gv_final=None):
        n = self.n
        gx = _f32(gx_final, (n, 3))
        gv = None if gv_final is None else _f32(gv_final, (n, 3))
        out = {k: np.empty(s, np.float32) for k, s in (("x", (n, 3)), ("v", (n, 3)), ("C", (n, 3, 3)), ("F", (n, 3, 3)))}
        pg = np.zeros(2, np.float64)
        _lib.check(self.L.mpm_diff_backward(self.h, _ptr(gx), _ptr(gv), _ptr(out["x"]), _ptr(out["v"]), _ptr(out["C"]),
                                            _ptr(out["F"]), _ptr(pg)))
        out["mu0"], out["lambda0"] = float(pg[0]), float(pg[1])
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.mpm_diff_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lame_grad(E: float, nu: float, gmu: float, glam: float):
    """Chain rule from (dL/dmu0, dL/dlambda0) to (dL/dE, dL/dnu) for
    mu0 = E / (2 (1 + nu)), lambda0 = E nu / ((1 + nu)(1 - 2 nu))."""
    dmu_dE = 1.0 / (2.0 * (1.0 + nu))
    dmu_dnu = -E / (2.0 * (1.0 + nu) ** 2)
    dlam_dE = nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    dlam_dnu = E * (1.0 + 2.0 * nu ** 2) / ((1.0 + nu) ** 2 * (1.0 - 2.0 * nu) ** 2)
    return gmu * dmu_dE + glam * dlam_dE, gmu * dmu_dnu + glam * dlam_dnu


class MPMRollout(torch.autograd.Function):
    """x_final = rollout(x0, v0, E, nu) over `nsteps` substeps of a DiffSim.

    Inputs are CPU tensors (float32 positions/velocities, scalar E and nu); the
    simulation itself runs on the GPU."""

    @staticmethod
    def forward(ctx, x0, v0, E, nu, sim: DiffSim, nsteps: int):
        sim.set_E_nu(float(E), float(nu))
        st = {"x": x0.detach().cpu().numpy(), "v": v0.detach().cpu().numpy()}
        xo, _ = sim.forward(st, int(nsteps))
        ctx.sim = sim
        ctx.E, ctx.nu = float(E), float(nu)
        return torch.from_numpy(xo)

    @staticmethod
    def backward(ctx, gx):
        g = ctx.sim.backward(gx.detach().cpu().numpy())
        gE, gnu = lame_grad(ctx.E, ctx.nu, g["mu0"], g["lambda0"])
        return (torch.from_numpy(g["x"]), torch.from_numpy(g["v"]), torch.tensor(gE, dtype=torch.float64),
                torch.tensor(gnu, dtype=torch.float64), None, None)


def rollout(x0, v0, E, nu, sim: DiffSim, nsteps: int):
    return MPMRollout.apply(x0, v0, E, nu, sim, nsteps)
