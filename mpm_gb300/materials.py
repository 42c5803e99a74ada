"""Material models behind the reference's MaterialModel interface.

The reference binds ``MaterialModel = MMSnow`` (include/mpm.cuh:25) and builds one
per ``[[material]]`` TOML table with ``MMSnow(1/particle_count, density, E, Nu,
hardening, plast_clamp_lower, plast_clamp_higher)`` (src/main.cu:34-47).  A
:class:`Material` carries the same constructor arguments plus the kind; the
derived constants (mass, mu0, lambda0) are computed in float32 exactly as the
reference constructors do (include/MaterialModel.cuh:26-29, 50-54).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SNOW, FIXED_COROTATED, JELLY, LIQUID = 0, 1, 2, 3
KIND_NAMES = {"snow": SNOW, "fixed_corotated": FIXED_COROTATED, "jelly": JELLY, "liquid": LIQUID}

f32 = np.float32


@dataclass
class Material:
    kind: int = SNOW
    particle_volume: float = 1.0 / 500000.0
    density: float = 400.0
    E: float = 1.4e5
    nu: float = 0.2
    hardening: float = 10.0
    clamp_lo: float = 1.0 - 2.5e-2
    clamp_hi: float = 1.0 + 7.5e-3
    bulk: float = 0.0
    name: str = field(default="", compare=False)

    def derived(self) -> dict:
        """Float32 constants exactly as MaterialModelBase / MMFixedCorotated compute them."""
        vol = f32(self.particle_volume)
        E, nu = f32(self.E), f32(self.nu)
        one, two = f32(1.0), f32(2.0)
        return {
            "kind": int(self.kind),
            "particle_volume": vol,
            "particle_mass": f32(f32(self.density) * vol),
            "mu0": f32(E / (two * (one + nu))),
            "lambda0": f32((E * nu) / ((one + nu) * (one - two * nu))),
            "hardening": f32(self.hardening),
            "clamp_lo": f32(self.clamp_lo),
            "clamp_hi": f32(self.clamp_hi),
            "bulk": f32(self.bulk),
        }


def snow(particle_volume, density=700.0, E=1.4e5, nu=0.2, hardening=10.0, theta_c=2.5e-2, theta_s=7.5e-3):
    """MMSnow with the snowman scene's parameters (scenes/snowman.toml)."""
    return Material(SNOW, particle_volume, density, E, nu, hardening, 1.0 - theta_c, 1.0 + theta_s, name="snow")


def elastic(particle_volume, density=1000.0, E=1e4, nu=0.3):
    """The reference's elastic ("rubber") material: MMSnow, hardening 0, clamps [0, 1e30]
    (scenes/rubber_duck.toml)."""
    return Material(SNOW, particle_volume, density, E, nu, 0.0, 0.0, 1.0e30, name="elastic")


def fixed_corotated(particle_volume, density=1000.0, E=1e4, nu=0.3):
    """MMFixedCorotated (no plasticity; stress uses Jp = 1)."""
    return Material(FIXED_COROTATED, particle_volume, density, E, nu, 0.0, 0.0, 1.0e30, name="fixed_corotated")


def liquid(particle_volume, density=1000.0, bulk=4e4):
    """Weakly compressible liquid: P F^T = K (J - 1) J I, J <- J det(I + dt C)."""
    return Material(LIQUID, particle_volume, density, 0.0, 0.0, 0.0, 0.0, 0.0, bulk, name="liquid")


def from_toml_table(table: dict, particle_count: float) -> Material:
    """One ``[[material]]`` table of a reference scene file, with the reference's
    defaults (src/main.cu:35-43) and ``particle_volume = 1/particle_count``."""
    kind = KIND_NAMES.get(str(table.get("kind", "snow")), SNOW)
    return Material(
        kind=kind,
        particle_volume=1.0 / float(particle_count),
        density=float(table.get("density", 700.0)),
        E=float(table.get("E", 1.4e5)),
        nu=float(table.get("Nu", 0.2)),
        hardening=float(table.get("hardening", 10.0)),
        clamp_lo=float(table.get("plast_clamp_lower", 0.975)),
        clamp_hi=float(table.get("plast_clamp_higher", 1.0075)),
        bulk=float(table.get("bulk", 0.0)),
        name=str(table.get("name", "")),
    )
