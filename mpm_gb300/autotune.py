"""Autotuner of the fused substep's launch shape (mpm_autotune in include/mpm_gb300.h).

The reference launches its kernels with a fixed 64-thread block per 64 particles
(src/mpm.cu:217-222).  Here the fused substep kernel has four knobs: the steps of 32
particles per range a warp claims, the CTA size (4, 6 or 12 warps), the G2P tile box
(4x4x6, 4x4x4 or 4x6x6 grid nodes) and the cell-sort interval.  :func:`tune` searches
them for a simulation's current scene on a device-side copy of its particles and applies
the winner; with a cache file, shapes found for the same device, library build and
workload class are reused without measuring.
"""
from __future__ import annotations

import ctypes
import os

from . import _lib

TILE_NAMES = {_lib.TILE_4x4x6: "4x4x6", _lib.TILE_4x4x4: "4x4x4", _lib.TILE_4x6x6: "4x6x6"}


def default_cache_path() -> str | None:
    """MPM_TUNING_CACHE when set, else None (no cache)."""
    return os.environ.get("MPM_TUNING_CACHE") or None


def _as_dict(t: _lib.MpmTuning) -> dict:
    return {"steps_per_warp": t.steps_per_warp, "warps_per_cta": t.warps_per_cta,
            "tile_box": TILE_NAMES.get(t.tile_box, t.tile_box), "sort_interval": t.sort_interval,
            "us_per_substep": t.us_per_substep, "from_cache": bool(t.from_cache), "candidates": t.candidates}


def tune(sim, cache_path: str | None = None, tune_sort_interval: bool = False, budget_substeps: int = 0,
         ignore_cache: bool = False) -> dict:
    """Chooses and applies the launch shape for `sim` (a Simulation with particles).
    Returns the chosen shape as a dict."""
    t = _lib.MpmTuning()
    flags = (_lib.TUNE_SORT_INTERVAL if tune_sort_interval else 0) | (_lib.TUNE_IGNORE_CACHE if ignore_cache else 0)
    path = cache_path.encode() if cache_path else None
    _lib.check(sim.L.mpm_autotune(sim.ctx, path, flags, int(budget_substeps), ctypes.byref(t)), sim.ctx)
    return _as_dict(t)


def current(sim) -> dict:
    """The simulation's current launch shape."""
    t = _lib.MpmTuning()
    _lib.check(sim.L.mpm_get_tuning(sim.ctx, ctypes.byref(t)), sim.ctx)
    return _as_dict(t)


def _batch_dict(t: _lib.MpmTuning) -> dict:
    return {"steps_per_warp": t.steps_per_warp, "warps_per_cta": t.warps_per_cta, "sort_interval": t.sort_interval,
            "us_per_substep": t.us_per_substep, "from_cache": bool(t.from_cache), "candidates": t.candidates}


def tune_batch(batch, cache_path: str | None = None, budget_substeps: int = 0, ignore_cache: bool = False,
               tune_sort_interval: bool = False) -> dict:
    """Chooses and applies the range size (steps per warp) of a Batch with particles, and
    with tune_sort_interval its sort interval, timed as replayed graphs on a copy of the
    batch (mpm_batch_autotune).  Returns the choice."""
    t = _lib.MpmTuning()
    flags = (_lib.TUNE_IGNORE_CACHE if ignore_cache else 0) | (_lib.TUNE_SORT_INTERVAL if tune_sort_interval else 0)
    path = cache_path.encode() if cache_path else None
    batch._check(batch.L.mpm_batch_autotune(batch.h, path, flags, int(budget_substeps), ctypes.byref(t)))
    return _batch_dict(t)


def current_batch(batch) -> dict:
    """The batch's current launch shape."""
    t = _lib.MpmTuning()
    batch._check(batch.L.mpm_batch_get_tuning(batch.h, ctypes.byref(t)))
    return _batch_dict(t)
