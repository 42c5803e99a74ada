"""Seeded synthetic scenes for the benchmark configurations.

The reference seeds particles with unseeded ``rand()`` and winding-number
rejection inside OBJ meshes (src/mpm.cu:10-12, 347-394); its meshes are not
available here.  These generators place particles uniformly in analytic boxes
and spheres with numpy's PCG64 generator, so the same seed gives the same state
on every machine.  Particle volume is the region volume divided by the count
(the reference's ``--particle-count`` is a density, include/options.h:29).
"""
from __future__ import annotations

import math

import numpy as np

from . import materials as M

GRAVITY = -9.8


def _empty_state(n: int) -> dict:
    eye = np.broadcast_to(np.eye(3, dtype=np.float32), (n, 3, 3)).copy()
    return {
        "x": np.zeros((n, 3), np.float32),
        "v": np.zeros((n, 3), np.float32),
        "C": np.zeros((n, 3, 3), np.float32),
        "F": eye,
        "Jp": np.ones(n, np.float32),
        "mat": np.zeros(n, np.uint8),
    }


def sample_box(rng, n, lo, hi):
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    return (lo + rng.random((n, 3)) * (hi - lo)).astype(np.float32)


def sample_sphere(rng, n, center, radius):
    out = np.empty((0, 3))
    c = np.asarray(center, np.float64)
    while out.shape[0] < n:
        pts = rng.random((max(2 * (n - out.shape[0]), 64), 3)) * 2.0 - 1.0
        pts = pts[np.einsum("ij,ij->i", pts, pts) <= 1.0]
        out = np.concatenate([out, pts], 0)
    return (c + radius * out[:n]).astype(np.float32)


def config_elastic(n=10_000, seed=0, N=16):
    """Plain elastic cube: N=16, particles U[0.35,0.65]^3, rho 1000, E 1e4, nu 0.3."""
    rng = np.random.default_rng(seed)
    st = _empty_state(n)
    st["x"] = sample_box(rng, n, (0.35,) * 3, (0.65,) * 3)
    vol = 0.3 ** 3 / n
    return {
        "name": "elastic",
        "state": st,
        "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3},
        "materials": [M.elastic(vol, density=1000.0, E=1e4, nu=0.3)],
        "substeps": 100,
    }


def config_liquid(n=1_000_000, seed=0, N=32):
    """Liquid throughput: N=32, particles U([0.1,0.5]x[0.1,0.7]x[0.1,0.9]), K 4e4."""
    rng = np.random.default_rng(seed)
    st = _empty_state(n)
    lo, hi = (0.1, 0.1, 0.1), (0.5, 0.7, 0.9)
    st["x"] = sample_box(rng, n, lo, hi)
    vol = 0.4 * 0.6 * 0.8 / n
    return {
        "name": "liquid",
        "state": st,
        "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3,
                   "sort_interval": 16},
        "materials": [M.liquid(vol, density=1000.0, bulk=4e4)],
        "substeps": 1000,
    }


def config_snow(n=500_000, seed=0, N=64):
    """Snow plasticity: two stacked spheres (r 0.15 at (0.5,0.3,0.5), r 0.1 at
    (0.5,0.55,0.5)), count split by volume, v0 = (0,-1,0)."""
    rng = np.random.default_rng(seed)
    r1, r2 = 0.15, 0.1
    v1, v2 = r1 ** 3, r2 ** 3
    n1 = int(round(n * v1 / (v1 + v2)))
    st = _empty_state(n)
    st["x"] = np.concatenate([sample_sphere(rng, n1, (0.5, 0.3, 0.5), r1),
                              sample_sphere(rng, n - n1, (0.5, 0.55, 0.5), r2)], 0)
    st["v"][:, 1] = -1.0
    vol = 4.0 / 3.0 * math.pi * (v1 + v2) / n
    return {
        "name": "snow",
        "state": st,
        "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3,
                   "sort_interval": 16},
        "materials": [M.snow(vol, density=700.0, E=1.4e5, nu=0.2, hardening=10.0)],
        "substeps": 500,
    }


def config_differentiable(n=100_000, seed=0, N=64):
    """Differentiable: fixed-corotated cube of side 0.2 centred at (0.5,0.6,0.5),
    v ~ N(0, 0.1^2) per component; 256 substeps, checkpoint every 16."""
    rng = np.random.default_rng(seed)
    st = _empty_state(n)
    st["x"] = sample_box(rng, n, (0.4, 0.5, 0.4), (0.6, 0.7, 0.6))
    st["v"] = (0.1 * rng.standard_normal((n, 3))).astype(np.float32)
    vol = 0.2 ** 3 / n
    return {
        "name": "differentiable",
        "state": st,
        "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3},
        "materials": [M.fixed_corotated(vol, density=1000.0, E=1e4, nu=0.3)],
        "substeps": 256,
        "target": np.array([0.6, 0.3, 0.5]),
        "checkpoint_every": 16,
    }


def mixed_scene(n=20_000, seed=0, N=32):
    """Several materials in one context (the reference's multi-material scenes)."""
    rng = np.random.default_rng(seed)
    n1 = n // 3
    n2 = n // 3
    n3 = n - n1 - n2
    st = _empty_state(n)
    st["x"] = np.concatenate([sample_box(rng, n1, (0.15, 0.2, 0.2), (0.35, 0.4, 0.4)),
                              sample_sphere(rng, n2, (0.6, 0.35, 0.5), 0.12),
                              sample_box(rng, n3, (0.4, 0.6, 0.3), (0.7, 0.75, 0.6))], 0)
    st["v"][:n1, 0] = 0.5
    st["mat"][n1:n1 + n2] = 1
    st["mat"][n1 + n2:] = 2
    vol = 1.0 / (n / 0.05)
    mats = [M.elastic(vol, density=1000.0, E=2e4, nu=0.3),
            M.snow(vol, density=700.0),
            M.liquid(vol, density=1000.0, bulk=2e4)]
    return {"name": "mixed", "state": st,
            "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3,
                       "sort_interval": 8},
            "materials": mats, "substeps": 100}


CONFIGS = {
    "elastic": config_elastic,
    "liquid": config_liquid,
    "snow": config_snow,
    "differentiable": config_differentiable,
}


def config_batched(nscenes=256, seed=0, count_range=(2_000, 200_000), grids=(16, 32, 64)):
    """Batched: independent scenes with log-uniform particle counts, N from {16,32,64},
    material from {elastic, liquid, snow} (the parameters of the plain scenes), a box
    or a sphere with a seeded random centre and size inside [0.1,0.9]^3; dt 1e-4."""
    rng = np.random.default_rng(seed)
    scenes = []
    lo, hi = np.log(count_range[0]), np.log(count_range[1])
    for i in range(nscenes):
        n = int(round(np.exp(rng.uniform(lo, hi))))
        N = int(rng.choice(grids))
        kind = int(rng.integers(0, 3))
        st = _empty_state(n)
        if rng.random() < 0.5:
            side = rng.uniform(0.1, 0.35, 3)
            c = rng.uniform(0.1 + side / 2, 0.9 - side / 2)
            st["x"] = sample_box(rng, n, c - side / 2, c + side / 2)
            vol_region = float(np.prod(side))
        else:
            r = rng.uniform(0.05, 0.18)
            c = rng.uniform(0.1 + r, 0.9 - r, 3)
            st["x"] = sample_sphere(rng, n, c, r)
            vol_region = 4.0 / 3.0 * math.pi * r ** 3
        vol = vol_region / n
        if kind == 0:
            mat = M.elastic(vol, density=1000.0, E=1e4, nu=0.3)
        elif kind == 1:
            mat = M.liquid(vol, density=1000.0, bulk=4e4)
        else:
            mat = M.snow(vol, density=700.0, E=1.4e5, nu=0.2, hardening=10.0)
            st["v"][:, 1] = -1.0
        scenes.append({"name": f"scene{i}", "state": st, "material": mat,
                       "params": {"dt": 1e-4, "N": N, "gravity": GRAVITY, "boundary_mode": 0, "boundary_cells": 3}})
    return scenes
