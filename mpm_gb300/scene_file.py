"""Scene objects and the reference's TOML scene files.

The reference builds a scene from a TOML file (src/main.cu:22-66): one ``[[material]]``
table per material, constructed as ``MMSnow(1 / particle_count, density, E, Nu,
hardening, plast_clamp_lower, plast_clamp_higher)`` with the defaults 700, 1.4e5, 0.2,
10, 0.975, 1.0075, and one ``[[object]]`` table per object, added with
``Simulation::addObject(mesh, material, size, position, velocity, lifetime_begin,
lifetime_end)`` (src/mpm.cu:237-251).  The scene's meshes live in a ``meshes/`` folder
beside the file.  Here:

* :class:`SceneObject` is one object: an analytic box or sphere, or a closed triangle
  mesh (read from an OBJ file), scaled so that its bounding box's longest edge is
  ``size``, with the box's lowest corner at ``position``.
* :func:`load_scene` reads a scene file into materials and objects.  ``cube.obj`` and
  ``sphere.obj`` map to the exact analytic box and sphere; any other mesh is read from
  the ``meshes/`` folder (:func:`read_obj`).
* :func:`build_simulation` creates a :class:`~mpm_gb300.simulation.Simulation` and adds
  the objects; their particles are seeded on the GPU (``mpm_add_object``) and join the
  simulation while ``lifetime_begin <= t < lifetime_end``.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .materials import SNOW, Material

try:  # Python 3.11+
    import tomllib as _toml
except ModuleNotFoundError:  # pragma: no cover
    _toml = None

FOREVER = 1e300

# MMSnow defaults of the scene reader (src/main.cu:35-43)
MATERIAL_DEFAULTS = {"density": 700.0, "E": 1.4e5, "Nu": 0.2, "hardening": 10.0, "plast_clamp_lower": 0.975,
                     "plast_clamp_higher": 1.0075}
# command-line defaults of the reference (include/options.h:25-29)
CLI_DEFAULTS = {"dt": 1e-4, "N": 60, "particle_count": 500000}


@dataclass
class SceneObject:
    shape: int = _lib.SHAPE_SPHERE
    material: int = 0
    size: float = 1.0
    position: tuple = (0.0, 0.0, 0.0)
    velocity: tuple = (0.0, 0.0, 0.0)
    box_extent: tuple = (1.0, 1.0, 1.0)
    lifetime_begin: float = 0.0
    lifetime_end: float = FOREVER
    seed: int = 0
    vertices: np.ndarray | None = None   # (V, 3) float32, MESH only
    triangles: np.ndarray | None = None  # (T, 3) int32, MESH only
    inside_test: int = _lib.INSIDE_RAY_PARITY  # MESH: _lib.INSIDE_WINDING for open meshes
    name: str = field(default="", compare=False)

    def to_c(self):
        """The mpm_object struct (keeps the mesh arrays alive on the returned holder)."""
        o = _lib.MpmObject()
        o.shape = int(self.shape)
        o.material = int(self.material)
        o.size = float(self.size)
        o.position[:] = [float(v) for v in self.position]
        o.velocity[:] = [float(v) for v in self.velocity]
        o.box_extent[:] = [float(v) for v in self.box_extent]
        o.lifetime_begin = float(self.lifetime_begin)
        o.lifetime_end = float(self.lifetime_end)
        o.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        o.inside_test = int(self.inside_test)
        keep = []
        if self.shape == _lib.SHAPE_MESH:
            V = np.ascontiguousarray(np.asarray(self.vertices, np.float32).reshape(-1, 3))
            T = np.ascontiguousarray(np.asarray(self.triangles, np.int32).reshape(-1, 3))
            keep = [V, T]
            o.vertices = V.ctypes.data_as(ctypes.c_void_p)
            o.n_vertices = V.shape[0]
            o.triangles = T.ctypes.data_as(ctypes.c_void_p)
            o.n_triangles = T.shape[0]
        return o, keep


def read_obj(path: str):
    """Vertices (V, 3) float32 and triangles (T, 3) int32 of an OBJ file; polygon faces
    are fanned into triangles, ``f`` indices may carry /texture/normal parts."""
    verts, tris = [], []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append([float(v) for v in parts[1:4]])
            elif parts[0] == "f":
                idx = [int(p.split("/")[0]) for p in parts[1:]]
                idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
                for k in range(1, len(idx) - 1):
                    tris.append([idx[0], idx[k], idx[k + 1]])
    if not verts or not tris:
        raise ValueError(f"{path}: no mesh (a Git LFS pointer file has no vertices)")
    return np.asarray(verts, np.float32), np.asarray(tris, np.int32)


def seed_object(obj: SceneObject, density: int) -> np.ndarray:
    """GPU seeding alone (mpm_seed_object): positions (n, 3) in candidate order."""
    L = _lib.lib()
    o, keep = obj.to_c()
    n = ctypes.c_int64()
    _lib.check(L.mpm_seed_object(ctypes.byref(o), int(density), None, 0, ctypes.byref(n)))
    x = np.empty((max(n.value, 1), 3), np.float32)
    _lib.check(L.mpm_seed_object(ctypes.byref(o), int(density), x.ctypes.data_as(ctypes.c_void_p), n.value,
                                 ctypes.byref(n)))
    del keep
    return x[:n.value]


def load_scene(path: str, particle_count: int = CLI_DEFAULTS["particle_count"], seed: int = 0):
    """Materials and objects of a reference scene file (src/main.cu:32-64)."""
    if _toml is None:  # pragma: no cover
        raise RuntimeError("tomllib is not available")
    with open(path, "rb") as f:
        cfg = _toml.load(f)
    mats, index = [], {}
    for i, t in enumerate(cfg.get("material", [])):
        g = lambda k: float(t.get(k, MATERIAL_DEFAULTS[k]))  # noqa: E731
        mats.append(Material(SNOW, 1.0 / float(particle_count), g("density"), g("E"), g("Nu"), g("hardening"),
                             g("plast_clamp_lower"), g("plast_clamp_higher"), name=str(t.get("name", ""))))
        index[str(t.get("name", ""))] = i
    meshes = os.path.join(os.path.dirname(os.path.abspath(path)), "meshes")
    objs = []
    for i, t in enumerate(cfg.get("object", [])):
        mesh = str(t.get("mesh", "sphere.obj"))
        o = SceneObject(material=index.get(str(t.get("material", "")), 0), size=float(t.get("size", 1.0)),
                        position=tuple(float(v) for v in t.get("position", [0, 0, 0])),
                        velocity=tuple(float(v) for v in t.get("velocity", [0, 0, 0])),
                        lifetime_begin=float(t.get("lifetime_begin", 0.0)),
                        lifetime_end=float(t.get("lifetime_end", FOREVER)), seed=seed * 1000003 + i, name=mesh)
        if mesh == "cube.obj":
            o.shape = _lib.SHAPE_BOX
        elif mesh == "sphere.obj":
            o.shape = _lib.SHAPE_SPHERE
        else:
            o.shape = _lib.SHAPE_MESH
            o.vertices, o.triangles = read_obj(os.path.join(meshes, mesh))
            # ray parity is exact for closed meshes; others take the winding number, the
            # reference's inside test (src/mpm.cu:383)
            if not is_closed(o.triangles):
                o.inside_test = _lib.INSIDE_WINDING
        objs.append(o)
    return mats, objs


def is_closed(triangles) -> bool:
    """Whether every edge of the triangle mesh is shared by exactly two triangles, in
    opposite directions (a closed, consistently oriented surface)."""
    T = np.asarray(triangles, np.int64).reshape(-1, 3)
    if T.size == 0:
        return False
    e = np.concatenate([T[:, [0, 1]], T[:, [1, 2]], T[:, [2, 0]]])
    key = lambda a, b: a * (int(T.max()) + 1) + b  # noqa: E731
    fwd, cnt = np.unique(key(e[:, 0], e[:, 1]), return_counts=True)
    if np.any(cnt != 1):
        return False
    rev = np.unique(key(e[:, 1], e[:, 0]))
    return len(fwd) == len(rev) and bool(np.all(fwd == rev))


def build_simulation(path: str, N: int = CLI_DEFAULTS["N"], dt: float = CLI_DEFAULTS["dt"],
                     particle_count: int = CLI_DEFAULTS["particle_count"], seed: int = 0, **params):
    """A Simulation with the scene's materials and objects (initCuda of src/main.cu:70)."""
    from .simulation import Simulation

    mats, objs = load_scene(path, particle_count, seed)
    sim = Simulation(dt=dt, N=N, **params)
    sim.set_materials(mats)
    for o in objs:
        sim.add_object(o)
    return sim
