"""Python wrapper of the batched-scenes C ABI (mpm_batch_* in include/mpm_gb300.h).

A batch advances many independent scenes — each with its own N, dt, material and
particle count — with one fused launch per substep for all of them, optionally as a
replayed CUDA graph.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .materials import Material


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _material(m: Material) -> _lib.MpmMaterial:
    return _lib.MpmMaterial(int(m.kind), float(m.particle_volume), float(m.density), float(m.E), float(m.nu),
                            float(m.hardening), float(m.clamp_lo), float(m.clamp_hi), float(m.bulk))


def _params(p: dict) -> _lib.MpmParams:
    return _lib.MpmParams(float(p["dt"]), int(p["N"]), float(p.get("gravity", -9.81)), int(p.get("boundary_mode", 0)),
                          int(p.get("boundary_cells", 3)), 0, 0, int(bool(p.get("check_finite", False))))


class Batch:
    """scenes: list of dicts with "params", "material" (Material) and "state" (or "count")."""

    def __init__(self, scenes, sort_interval=16):
        self.L = _lib.lib()
        arr = (_lib.MpmScene * len(scenes))()
        for i, sc in enumerate(scenes):
            count = int(sc["state"]["x"].shape[0]) if "state" in sc else int(sc["count"])
            arr[i] = _lib.MpmScene(_params(sc["params"]), _material(sc["material"]), count)
        h = ctypes.c_void_p()
        code = self.L.mpm_batch_create(arr, len(scenes), int(sort_interval), ctypes.byref(h))
        if code != 0:
            raise _lib.MpmError(code, "mpm_batch_create failed")
        self.h = h
        self.counts = [int(arr[i].count) for i in range(len(scenes))]
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        self.n = int(self.offsets[-1])

    def _check(self, code):
        if code != 0:
            buf = ctypes.create_string_buffer(512)
            self.L.mpm_batch_last_error(self.h, buf, 512)
            raise _lib.MpmError(code, buf.value.decode(errors="replace"))

    def set_stream(self, handle: int):
        self._check(self.L.mpm_batch_set_stream(self.h, ctypes.c_void_p(int(handle))))

    def set_steps_per_warp(self, steps_per_warp: int):
        """Range size of the batched kernel in 32-particle steps (1..256)."""
        self._check(self.L.mpm_batch_set_steps_per_warp(self.h, int(steps_per_warp)))

    def set_sort_interval(self, sort_interval: int):
        """Substeps between cell sorts (0: never)."""
        self._check(self.L.mpm_batch_set_sort_interval(self.h, int(sort_interval)))

    def upload(self, states):
        """states: one state dict per scene (or one concatenated dict)."""
        if isinstance(states, dict):
            cat = states
        else:
            cat = {k: np.concatenate([np.asarray(s[k], np.float32).reshape(len(s["x"]), -1) for s in states], 0)
                   for k in ("x", "v", "C", "F", "Jp")}
        n = self.n
        a = {k: np.ascontiguousarray(np.asarray(cat[k], np.float32).reshape(n, -1)) for k in ("x", "v", "C", "F", "Jp")}
        self._check(self.L.mpm_batch_upload_soa(self.h, _ptr(a["x"]), _ptr(a["v"]), _ptr(a["C"]), _ptr(a["F"]),
                                                _ptr(a["Jp"])))

    def advance(self, nsteps=1, graph=False):
        fn = self.L.mpm_batch_substep_graph if graph else self.L.mpm_batch_substep
        self._check(fn(self.h, int(nsteps)))

    def sync(self):
        self._check(self.L.mpm_batch_sync(self.h))

    def download(self):
        n = self.n
        out = {"x": np.empty((n, 3), np.float32), "v": np.empty((n, 3), np.float32),
               "C": np.empty((n, 3, 3), np.float32), "F": np.empty((n, 3, 3), np.float32),
               "Jp": np.empty((n,), np.float32)}
        self._check(self.L.mpm_batch_download_soa(self.h, _ptr(out["x"]), _ptr(out["v"]), _ptr(out["C"]),
                                                  _ptr(out["F"]), _ptr(out["Jp"])))
        return out

    def split(self, cat):
        """Concatenated state -> list of per-scene states."""
        return [{k: v[self.offsets[i]:self.offsets[i + 1]] for k, v in cat.items()} for i in range(len(self.counts))]

    @property
    def launches(self):
        return int(self.L.mpm_batch_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.mpm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
