"""GPU tests of material models compiled into the substep kernel through the public
policy header (include/mpm_gb300_policies.cuh; the reference's compile-time MaterialModel
alias, include/mpm.cuh:25).  The test translation unit tests/plugin_materials.cu defines,
through that header only, kind 16 (the reference's MMJelly) and kind 17 (MMJelly with twice
the shear modulus); a build of the library with it runs them in the fused substep kernel.

Bar: the oracle's MMJelly (FP32) within 1e-5 after 3 substeps, as the built-in models are
held in tests/test_gpu_parity.py; kind 17 against the oracle's MMJelly with mu0 doubled."""
import os

import numpy as np
import pytest

from helpers import compare_states

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def plugin_lib(gpu_lib, tmp_path_factory):
    from mpm_gb300 import _lib, build

    out = str(tmp_path_factory.mktemp("plugin") / "libmpm_gb300_plugins.so")
    return _lib.load_library(build.build_with_materials([os.path.join(HERE, "plugin_materials.cu")], out))


def jelly_scene(kind, seed=41, n=30_000, N=32):
    """A jelly block with a spin and a compression, heavy enough that the stress matters."""
    from mpm_gb300 import scenes
    from mpm_gb300.materials import JELLY, Material

    rng = np.random.default_rng(seed)
    st = scenes._empty_state(n)
    lo, hi = np.array([0.35, 0.4, 0.35]), np.array([0.65, 0.6, 0.65])
    x = scenes.sample_box(rng, n, lo, hi).astype(np.float64)
    c = x.mean(0)
    st["x"] = x.astype(np.float32)
    st["v"] = (np.cross([0.0, 3.0, 0.0], x - c) - 2.0 * (x - c)).astype(np.float32)
    st["Jp"] = rng.uniform(0.9, 1.1, n).astype(np.float32)
    vol = float(np.prod(hi - lo)) / n
    mat = Material(kind, vol, 1000.0, 2e5, 0.3, 5.0, 0.0, 1e30, 0.0, name=f"jelly{kind}")
    ref_mat = Material(JELLY, vol, 1000.0, 2e5, 0.3, 5.0, 0.0, 1e30, 0.0, name="jelly")
    params = {"dt": 1e-4, "N": N, "gravity": -9.8, "boundary_mode": 0, "boundary_cells": 3, "sort_interval": 2}
    return st, params, mat, ref_mat


def run_plugin(L, st, params, mat, nsteps):
    from mpm_gb300.simulation import Simulation

    with Simulation(library=L, materials=[mat], **params) as sim:
        sim.upload(st)
        sim.advance(nsteps)
        return sim.syncDevice()


@pytest.mark.parametrize("kind,mu_scale", [(16, 1.0), (17, 2.0)])
def test_compiled_in_material_matches_oracle(plugin_lib, oracle_lib, kind, mu_scale):
    st, params, mat, ref_mat = jelly_scene(kind)
    out = run_plugin(plugin_lib, st, params, mat, 3)
    d = ref_mat.derived()
    d["mu0"] = float(np.float32(mu_scale * np.float32(d["mu0"])))
    ref, _, _ = oracle_lib.substep(st, params, [d], 3, np.float32)
    errs = compare_states(out, ref, params, st)
    assert max(errs.values()) < 1e-5, errs


def test_compiled_in_materials_differ(plugin_lib):
    """The kernel runs the plug-in's code: after 3 substeps the two models' velocities
    differ by more than 1e-4 of their largest value, ten times the parity bar (3.5e-4 was
    measured on GB300)."""
    st, params, m16, _ = jelly_scene(16)
    _, _, m17, _ = jelly_scene(17)
    a = run_plugin(plugin_lib, st, params, m16, 3)
    b = run_plugin(plugin_lib, st, params, m17, 3)
    assert np.abs(a["v"] - b["v"]).max() > 1e-4 * np.abs(a["v"]).max()


def test_material_tables_are_checked(plugin_lib, gpu_lib):
    from mpm_gb300 import _lib
    from mpm_gb300.materials import SNOW, Material
    from mpm_gb300.simulation import Simulation

    st, params, m16, _ = jelly_scene(16, n=1000)
    snow = Material(SNOW, m16.particle_volume, 700.0, 1.4e5, 0.2, 10.0, 0.975, 1.0075, 0.0)
    unknown = Material(18, m16.particle_volume, 1000.0, 2e5, 0.3, 5.0, 0.0, 1e30, 0.0)
    with Simulation(library=plugin_lib, **params) as sim:
        with pytest.raises(_lib.MpmError):
            sim.set_materials([unknown])  # not compiled in
        with pytest.raises(_lib.MpmError):
            sim.set_materials([m16, snow])  # a compiled-in kind holds its table alone
        sim.set_materials([m16, m16])
    with Simulation(**params) as sim:  # the package's own build has no kind 16
        with pytest.raises(_lib.MpmError):
            sim.set_materials([m16])
