"""GPU test of mpm_substep_noalloc, the substep entry point that allocates nothing.

Callers that cannot call cudaMalloc use this entry point: plugins whose host
application owns all device memory through its own pool, and embedded or real-time
callers that forbid allocation after start-up.  They pass their own device buffers for
the particle state; the substep's scratch (the rotating P2G grids, the velocity grid
and the device status word) is a static device array inside the library, limited to
N <= 32.  mpm_noalloc_status reads and clears that status word.

The file is named so that pytest collects it last: a run that stops at the first
failure has already run every other test.  Each check compares the entry point with
the context path (mpm_upload_soa + mpm_substep + mpm_download_soa) on the same
state, within the 1e-5 parity tolerance of the other GPU tests, over two calls in a
row (the second call reuses the scratch the first one left behind).
"""
import ctypes

import numpy as np
import pytest

from helpers import compare_states

pytestmark = pytest.mark.gpu

NCOMP = 25  # x 0-2, v 3-5, C 6-14, F 15-23, Jp 24


def to_component_major(state, stride):
    n = state["x"].shape[0]
    buf = np.zeros((NCOMP, stride), np.float32)
    buf[0:3, :n] = state["x"].T
    buf[3:6, :n] = state["v"].T
    buf[6:15, :n] = state["C"].reshape(n, 9).T
    buf[15:24, :n] = state["F"].reshape(n, 9).T
    buf[24, :n] = state["Jp"]
    return buf


def from_component_major(buf, n):
    return {"x": buf[0:3, :n].T.copy(), "v": buf[3:6, :n].T.copy(), "C": buf[6:15, :n].T.reshape(n, 3, 3).copy(),
            "F": buf[15:24, :n].T.reshape(n, 3, 3).copy(), "Jp": buf[24, :n].copy()}


def scenes_under_test():
    from mpm_gb300 import scenes

    return {
        "elastic_N16": scenes.config_elastic(n=10_000, seed=21),
        "liquid_N32": scenes.config_liquid(n=120_000, seed=22),
        "snow_N32": scenes.config_snow(n=80_000, seed=23, N=32),
        "mixed_N32": scenes.mixed_scene(n=20_000, seed=24),
    }


def call_noalloc(L, cfg, dev_state, stride, dev_mat, n, nsteps):
    import torch

    from mpm_gb300 import _lib

    p = cfg["params"]
    params = _lib.MpmParams(float(p["dt"]), int(p["N"]), float(p.get("gravity", -9.81)), int(p.get("boundary_mode", 0)),
                            int(p.get("boundary_cells", 3)), 0, 0, 0)
    mats = (_lib.MpmMaterial * len(cfg["materials"]))()
    for i, m in enumerate(cfg["materials"]):
        mats[i] = _lib.MpmMaterial(int(m.kind), float(m.particle_volume), float(m.density), float(m.E), float(m.nu),
                                   float(m.hardening), float(m.clamp_lo), float(m.clamp_hi), float(m.bulk))
    rc = L.mpm_substep_noalloc(ctypes.byref(params), mats, len(cfg["materials"]), ctypes.c_void_p(dev_state.data_ptr()),
                               stride, ctypes.c_void_p(dev_mat.data_ptr()) if dev_mat is not None else None, n, nsteps,
                               None)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("name", list(scenes_under_test().keys()))
def test_noalloc_matches_context_path(gpu_lib, name):
    import torch

    from mpm_gb300.simulation import Simulation

    cfg = scenes_under_test()[name]
    st = cfg["state"]
    n = st["x"].shape[0]
    liquid = len(cfg["materials"]) == 1 and cfg["materials"][0].kind == 3

    with Simulation.from_config(cfg, sort_interval=0) as sim:
        sim.upload(st)
        sim.advance(2)
        ref1 = sim.syncDevice()
        sim.advance(3)
        ref2 = sim.syncDevice()

    stride = (n + 63) // 64 * 64
    dev = torch.from_numpy(to_component_major(st, stride)).cuda()
    dev_mat = torch.from_numpy(np.ascontiguousarray(st["mat"])).cuda() if len(cfg["materials"]) > 1 else None
    fields = ("x", "v", "C", "Jp") if liquid else ("x", "v", "C", "F", "Jp")

    assert call_noalloc(gpu_lib, cfg, dev, stride, dev_mat, n, 2) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 0
    out1 = from_component_major(dev.cpu().numpy(), n)
    errs = compare_states(out1, ref1, cfg["params"], st)
    assert max(errs[k] for k in fields) < 1e-5, errs

    assert call_noalloc(gpu_lib, cfg, dev, stride, dev_mat, n, 3) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 0
    out2 = from_component_major(dev.cpu().numpy(), n)
    errs = compare_states(out2, ref2, cfg["params"], st)
    assert max(errs[k] for k in fields) < 1e-5, errs


def test_noalloc_rejects_grid_beyond_scratch(gpu_lib):
    """N above the static scratch's 32 is refused with MPM_ERR_UNSUPPORTED, before any launch."""
    import torch

    from mpm_gb300 import scenes

    cfg = scenes.config_snow(n=2_000, seed=25, N=64)
    st = cfg["state"]
    dev = torch.from_numpy(to_component_major(st, 2048)).cuda()
    before = dev.clone()
    assert call_noalloc(gpu_lib, cfg, dev, 2048, None, 2_000, 1) == 6
    assert torch.equal(dev, before)


def test_noalloc_status_reports_an_expired_wait(gpu_lib):
    """A bounded device wait that runs out sets the no-allocation status word: a warp
    waits on an mbarrier that nothing completes and gives up after 64 polls, as the
    substep does when a tile copy never lands.  The bit survives a following substep
    call (which does not clear it), mpm_noalloc_status returns MPM_ERR_TIMEOUT once and
    clears it, and the substeps keep working afterwards."""
    import torch

    from mpm_gb300 import scenes

    assert gpu_lib.mpm_noalloc_status(None) == 0
    assert gpu_lib.mpm_noalloc_check_wait_timeout(0, None) == 1  # polls out of range
    assert gpu_lib.mpm_noalloc_check_wait_timeout(64, None) == 0
    cfg = scenes.config_elastic(n=4_000, seed=26)
    st = cfg["state"]
    dev = torch.from_numpy(to_component_major(st, 4032)).cuda()
    assert call_noalloc(gpu_lib, cfg, dev, 4032, None, 4_000, 1) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 4  # MPM_ERR_TIMEOUT
    assert gpu_lib.mpm_noalloc_status(None) == 0  # cleared by the read
    assert call_noalloc(gpu_lib, cfg, dev, 4032, None, 4_000, 1) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 0
    assert torch.isfinite(dev).all()


def test_noalloc_flags_material_index_past_the_table(gpu_lib):
    """A material index the table does not hold is flagged (MPM_ERR_STATE) and the
    particle takes material 0, so the result equals that of an all-zero material array
    (to the rounding of the grid's float atomics, whose order varies between runs)."""
    import torch

    from mpm_gb300 import scenes

    cfg = scenes.mixed_scene(n=6_000, seed=27)
    st = cfg["state"]
    n = st["x"].shape[0]
    stride = (n + 63) // 64 * 64
    zero = torch.zeros(n, dtype=torch.uint8, device="cuda")
    bad = zero.clone()
    bad[n // 2] = 200
    a = torch.from_numpy(to_component_major(st, stride)).cuda()
    b = a.clone()
    assert gpu_lib.mpm_noalloc_status(None) == 0
    assert call_noalloc(gpu_lib, cfg, a, stride, zero, n, 2) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 0
    assert call_noalloc(gpu_lib, cfg, b, stride, bad, n, 2) == 0
    assert gpu_lib.mpm_noalloc_status(None) == 3  # MPM_ERR_STATE
    n_ = st["x"].shape[0]
    errs = compare_states(from_component_major(b.cpu().numpy(), n_), from_component_major(a.cpu().numpy(), n_),
                          cfg["params"], st)
    assert max(errs.values()) < 1e-5, errs
