"""Python mirror of the reference's ``Simulation`` host class.

``Simulation`` (include/mpm.cuh:44-106, src/mpm.cu:180-329) keeps the same method
names — ``initCuda``, ``advance``, ``syncDevice``, ``getFullParticleCount`` — on
top of the C ABI in include/mpm_gb300.h.  Errors are raised as
:class:`mpm_gb300._lib.MpmError` with the library's message (the reference calls
``exit()`` or does not check).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .materials import Material


def _f32(a, shape):
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shape))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Simulation:
    """One simulation context on the current CUDA device.

    Parameters mirror ``SimulationParameters`` (dt, N) plus the options the
    reference hard-codes (gravity -9.81, the 0.05 boundary fraction) and the
    sort interval of the cell-sorted layout."""

    def __init__(self, dt=1e-4, N=60, gravity=-9.81, boundary_mode=0, boundary_cells=3, g2p_guard=False,
                 sort_interval=16, check_finite=False, materials=None, library=None):
        # library: a build with compiled-in material models (_lib.load_library); default:
        # the library of this package
        self.L = library if library is not None else _lib.lib()
        self.params = _lib.MpmParams(float(dt), int(N), float(gravity), int(boundary_mode), int(boundary_cells),
                                     int(bool(g2p_guard)), int(sort_interval), int(bool(check_finite)))
        ctx = ctypes.c_void_p()
        code = self.L.mpm_create(ctypes.byref(self.params), ctypes.byref(ctx))
        if code != 0:
            raise _lib.MpmError(code, "mpm_create failed")
        self.ctx = ctx
        _lib.register_context(ctx, self.L)
        self.N = int(N)
        self.materials = []
        if materials is not None:
            self.set_materials(materials)

    @classmethod
    def from_config(cls, cfg: dict, **overrides):
        p = dict(cfg["params"])
        p.update(overrides)
        sim = cls(**p)
        sim.set_materials(cfg["materials"])
        return sim

    # -- setup -------------------------------------------------------------
    def set_materials(self, materials):
        arr = (_lib.MpmMaterial * len(materials))()
        for i, m in enumerate(materials):
            if not isinstance(m, Material):
                raise TypeError("materials must be mpm_gb300.materials.Material")
            arr[i] = _lib.MpmMaterial(int(m.kind), float(m.particle_volume), float(m.density), float(m.E),
                                      float(m.nu), float(m.hardening), float(m.clamp_lo), float(m.clamp_hi),
                                      float(m.bulk))
        _lib.check(self.L.mpm_set_materials(self.ctx, arr, len(materials)), self.ctx)
        self.materials = list(materials)

    def set_params(self, **kw):
        for k, v in kw.items():
            setattr(self.params, k, v)
        _lib.check(self.L.mpm_set_params(self.ctx, ctypes.byref(self.params)), self.ctx)

    def set_stream(self, handle):
        """Enqueue all further work on the cudaStream_t `handle` (an int; 0 = the context's own)."""
        _lib.check(self.L.mpm_set_stream(self.ctx, ctypes.c_void_p(int(handle)) if handle else None), self.ctx)

    def set_tuning(self, steps_per_warp=0, warps_per_cta=0, tile_box=0):
        """Fused-kernel knobs (0 keeps the current value): 32-particle steps per range a warp
        claims, warps per CTA (4, 6 or 12) and the G2P tile box (_lib.TILE_*)."""
        _lib.check(self.L.mpm_set_tuning(self.ctx, int(steps_per_warp), int(warps_per_cta), int(tile_box)),
                   self.ctx)

    def upload(self, state: dict):
        """particlesToDevice (src/mpm.cu:278-286): x, v, C, F, Jp, mat host arrays."""
        n = int(np.asarray(state["x"]).shape[0])
        x = _f32(state["x"], (n, 3))
        v = _f32(state.get("v"), (n, 3))
        C = _f32(state.get("C"), (n, 9))
        F = _f32(state.get("F"), (n, 9))
        J = _f32(state.get("Jp"), (n,))
        mat = state.get("mat")
        if mat is not None:
            mat = np.ascontiguousarray(np.asarray(mat, dtype=np.uint8).reshape(n))
        _lib.check(self.L.mpm_upload_soa(self.ctx, n, _ptr(x), _ptr(v), _ptr(C), _ptr(F), _ptr(J), _ptr(mat)),
                   self.ctx)

    initCuda = upload

    def upload_aos(self, records: np.ndarray):
        """Upload the reference's 104-byte MLS_APIC_Particle records."""
        rec = np.ascontiguousarray(records)
        n = rec.nbytes // 104
        _lib.check(self.L.mpm_upload_aos(self.ctx, _ptr(rec), n), self.ctx)

    # -- scene objects -----------------------------------------------------
    def add_object(self, obj) -> int:
        """Simulation::addObject (src/mpm.cu:237-251): seed a
        :class:`mpm_gb300.scene_file.SceneObject` on the GPU; its particles join the
        simulation while lifetime_begin <= t < lifetime_end.  Returns its particle count."""
        o, keep = obj.to_c()
        count = ctypes.c_int64()
        _lib.check(self.L.mpm_add_object(self.ctx, ctypes.byref(o), ctypes.byref(count)), self.ctx)
        del keep
        return int(count.value)

    @property
    def t(self) -> float:
        """Simulated time (Simulation::t)."""
        return float(self.L.mpm_time(self.ctx))

    @property
    def object_count(self) -> int:
        return int(self.L.mpm_object_count(self.ctx))

    @property
    def n(self) -> int:
        """Particles currently simulated (uploaded plus active objects)."""
        return int(self.L.mpm_particle_count(self.ctx))

    # -- stepping ----------------------------------------------------------
    def advance(self, nsteps: int = 1):
        """Simulation::advance (src/mpm.cu:323-329), nsteps times, asynchronous."""
        _lib.check(self.L.mpm_substep(self.ctx, int(nsteps)), self.ctx)

    def sync(self):
        _lib.check(self.L.mpm_sync(self.ctx), self.ctx)

    def sort(self):
        _lib.check(self.L.mpm_sort(self.ctx), self.ctx)

    # -- readback ----------------------------------------------------------
    def download(self, fields=("x", "v", "C", "F", "Jp", "mat")) -> dict:
        n = self.n
        out = {
            "x": np.empty((n, 3), np.float32) if "x" in fields else None,
            "v": np.empty((n, 3), np.float32) if "v" in fields else None,
            "C": np.empty((n, 3, 3), np.float32) if "C" in fields else None,
            "F": np.empty((n, 3, 3), np.float32) if "F" in fields else None,
            "Jp": np.empty((n,), np.float32) if "Jp" in fields else None,
            "mat": np.empty((n,), np.uint8) if "mat" in fields else None,
        }
        _lib.check(self.L.mpm_download_soa(self.ctx, _ptr(out["x"]), _ptr(out["v"]), _ptr(out["C"]),
                                           _ptr(out["F"]), _ptr(out["Jp"]), _ptr(out["mat"])), self.ctx)
        return {k: v for k, v in out.items() if v is not None}

    def syncDevice(self) -> dict:
        """Simulation::syncDevice (src/mpm.cu:209-211): blocking readback of all particles."""
        self.sync()
        return self.download()

    def download_aos(self) -> np.ndarray:
        out = np.zeros(self.n * 104, np.uint8)
        _lib.check(self.L.mpm_download_aos(self.ctx, _ptr(out)), self.ctx)
        return out

    def get_grid(self, which: int = 0) -> np.ndarray:
        """Grid of the last completed substep: 0 = after P2G (m v, m), 1 = after the grid op."""
        out = np.empty((self.N, self.N, self.N, 4), np.float32)
        _lib.check(self.L.mpm_get_grid(self.ctx, int(which), _ptr(out)), self.ctx)
        return out

    # -- surface reconstruction ------------------------------------------
    def surface_distance(self, grid_side: int = 250, radius: int = 5) -> np.ndarray:
        """Distance field (G, G, G) float32 of fillVoxelGrid_distance
        (include/mesh_builder.h:89-137) on the voxel grid of MeshBuilder::computeMesh."""
        G = int(grid_side)
        out = np.empty((G, G, G), np.float32)
        _lib.check(self.L.mpm_surface_distance(self.ctx, G, int(radius), _ptr(out)), self.ctx)
        return out

    def surface_indexed(self, grid_side: int = 250, radius: int = 5):
        """The particles' surface as MeshBuilder::computeMesh hands it to igl::writeOBJ
        (include/mesh_builder.h:170-210): vertices (V, 3) float64 in libigl's marching-cubes
        order, bit for bit, and outward faces (F, 3) int32 (zero-based)."""
        G = int(grid_side)
        nv, nf = ctypes.c_int64(), ctypes.c_int64()
        # a first guess of the sizes (a surface crossing 16 G^2 cubes); retried once if short
        guess = max(1, min(5 * (G - 1) ** 3, 16 * G * G))
        V = np.empty((guess, 3), np.float64)
        F = np.empty((guess, 3), np.int32)
        _lib.check(self.L.mpm_surface_mesh_indexed(self.ctx, G, int(radius), _ptr(V), V.shape[0], _ptr(F), F.shape[0],
                                                   ctypes.byref(nv), ctypes.byref(nf)), self.ctx)
        if nv.value > V.shape[0] or nf.value > F.shape[0]:
            V = np.empty((max(nv.value, 1), 3), np.float64)
            F = np.empty((max(nf.value, 1), 3), np.int32)
            _lib.check(self.L.mpm_surface_mesh_indexed(self.ctx, G, int(radius), _ptr(V), V.shape[0], _ptr(F),
                                                       F.shape[0], ctypes.byref(nv), ctypes.byref(nf)), self.ctx)
        return V[:nv.value], F[:nf.value]

    def smooth_mesh(self, V: np.ndarray, F: np.ndarray) -> np.ndarray:
        """MeshBuilder::smoothMesh (include/mesh_builder.h:212-245) on the GPU: one implicit
        cotangent-Laplacian smoothing step (M - 0.001 L) U = M V, rescaled to unit area
        (mpm_surface_smooth); returns U (V, 3) float64."""
        U = np.ascontiguousarray(np.asarray(V, np.float64).reshape(-1, 3)).copy()
        Fi = np.ascontiguousarray(np.asarray(F, np.int32).reshape(-1, 3))
        it = ctypes.c_int32()
        _lib.check(self.L.mpm_surface_smooth(self.ctx, _ptr(U), U.shape[0], _ptr(Fi), Fi.shape[0], ctypes.byref(it)),
                   self.ctx)
        self.smooth_iterations = it.value
        return U

    def surface_mesh(self, grid_side: int = 250, radius: int = 5) -> np.ndarray:
        """Triangles (T, 3, 3) float32 of the particles' surface (the zero level of
        radius voxel_dx - distance, include/mesh_builder.h:170-190): the faces of
        surface_indexed with their vertices rounded to float, in the same order."""
        G = int(grid_side)
        n = ctypes.c_int64()
        # a first guess of the triangle count (a surface crossing 16 G^2 cells); retried once if short
        out = np.empty((max(1, min(5 * (G - 1) ** 3, 16 * G * G)), 3, 3), np.float32)
        _lib.check(self.L.mpm_surface_mesh(self.ctx, G, int(radius), _ptr(out), out.shape[0], ctypes.byref(n)),
                   self.ctx)
        if n.value > out.shape[0]:
            out = np.empty((n.value, 3, 3), np.float32)
            _lib.check(self.L.mpm_surface_mesh(self.ctx, G, int(radius), _ptr(out), n.value, ctypes.byref(n)),
                       self.ctx)
        return out[:n.value]

    def getFullParticleCount(self) -> int:
        return int(self.L.mpm_particle_count(self.ctx))

    @property
    def substeps(self) -> int:
        return int(self.L.mpm_substep_count(self.ctx))

    @property
    def launches(self) -> int:
        return int(self.L.mpm_launch_count(self.ctx))

    def close(self):
        if getattr(self, "ctx", None):
            _lib.forget_context(self.ctx)
            self.L.mpm_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def advance_many(sims, nsteps: int = 1):
    """Simulation::advance over several independent scenes: nsteps substeps of every
    simulation, interleaved substep by substep, in one compiled loop (mpm_substep_many)."""
    sims = list(sims)
    if not sims:
        return
    L = sims[0].L
    arr = (ctypes.c_void_p * len(sims))(*[s.ctx.value for s in sims])
    code = L.mpm_substep_many(arr, len(sims), int(nsteps))
    if code != 0:
        for s in sims:  # report the context that failed, when it recorded a message
            buf = ctypes.create_string_buffer(512)
            L.mpm_last_error(s.ctx, buf, 512)
            if buf.value:
                raise _lib.MpmError(code, buf.value.decode(errors="replace"))
        raise _lib.MpmError(code, "mpm_substep_many failed")
