"""mpm_gb300 — MLS-MPM substep for NVIDIA GB300 (sm_103a).

Drop-in for the substep of kekeblom/mpm behind its MaterialModel /
TransferScheme / InterpolationKernel interfaces.  The compute path is the CUDA
library ``libmpm_gb300.so`` (C ABI in include/mpm_gb300.h); this package holds
the host-side mirror of the reference's ``Simulation`` class, the material
definitions and the seeded scene generators.
"""
from . import materials, scenes  # noqa: F401
from .materials import Material  # noqa: F401

__all__ = ["materials", "scenes", "Material", "Simulation", "build"]


def __getattr__(name):
    if name == "Simulation":
        from .simulation import Simulation

        return Simulation
    if name == "build":
        from .build import build

        return build
    raise AttributeError(name)
