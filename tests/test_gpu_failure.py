"""Failure detection on the GPU without a GPU fault: every wait of the substep kernel is
bounded and reports through the status word.  The check makes one such wait run out
(an mbarrier nothing arrives on) and expects MPM_ERR_TIMEOUT from mpm_sync, then a
normal substep on the same context."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives(gpu_lib, oracle_lib):
    from helpers import compare_states
    from mpm_gb300 import _lib, scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=2000, seed=11)
    with Simulation.from_config(cfg) as sim:
        code = gpu_lib.mpm_check_wait_timeout(sim.ctx, 1000)
        assert _lib.STATUS_NAMES[code] == "MPM_ERR_TIMEOUT"
        # the status word was read and cleared: the context keeps working
        sim.upload(cfg["state"])
        sim.advance(2)
        out = sim.syncDevice()
    mats = [m.derived() for m in cfg["materials"]]
    o32, _, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, 2, np.float32)
    errs = compare_states(out, o32, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs


def test_wait_check_rejects_bad_limits(gpu_lib):
    from mpm_gb300 import _lib, scenes
    from mpm_gb300.simulation import Simulation

    cfg = scenes.config_elastic(n=100, seed=1)
    with Simulation.from_config(cfg) as sim:
        assert _lib.STATUS_NAMES[gpu_lib.mpm_check_wait_timeout(sim.ctx, 0)] == "MPM_ERR_INVALID"
        assert _lib.STATUS_NAMES[gpu_lib.mpm_check_wait_timeout(sim.ctx, 1 << 21)] == "MPM_ERR_INVALID"
