"""Surface meshes of the particles: the reference's MeshBuilder (include/mesh_builder.h).

``MeshBuilder(N, dx, grid_side, particle_radius).computeMesh(filename, sim)`` follows
MeshBuilder::computeMesh (include/mesh_builder.h:170-211) as src/main.cu:78-106 drives it
once per saved frame: the distance field and the marching-cubes mesh are computed on the
GPU (``mpm_surface_mesh_indexed``: libigl's vertex list bit for bit, faces over the same
edge loops) and written as an OBJ file (igl::writeOBJ's ``v`` / ``f`` lines).  ``laplacian_smooth``
(the reference's ``--laplacian_smooth``, off by default) applies MeshBuilder::smoothMesh
(include/mesh_builder.h:212-245) on the GPU (``mpm_surface_smooth``): one implicit
cotangent-Laplacian step and the rescale to unit area.  The reference's other optional
post-processing step, ``--mesh-face-count`` decimation by igl::decimate (off by default),
is not provided.
"""
from __future__ import annotations

import numpy as np

# command-line defaults of the reference (include/options.h:30-31)
MESH_GRID = 250
MESH_PARTICLE_RADIUS = 5


def weld(tris: np.ndarray):
    """Indexed mesh (V (n, 3), F (T, 3) int32) of a triangle soup (T, 3, 3), for soups
    from mpm_surface_mesh.  Vertices on the same voxel edge are bit-identical, so exact
    matching welds them.  Where the level set passes exactly through a voxel node, edge
    points coincide and their triangles collapse to a repeated index; those faces are
    dropped."""
    pts = np.ascontiguousarray(tris.reshape(-1, 3))
    if pts.shape[0] == 0:
        return np.zeros((0, 3), pts.dtype), np.zeros((0, 3), np.int32)
    V, inv = np.unique(pts.view(np.dtype((np.void, 3 * pts.itemsize))).ravel(), return_inverse=True)
    F = inv.reshape(-1, 3).astype(np.int32)
    F = F[(F[:, 0] != F[:, 1]) & (F[:, 1] != F[:, 2]) & (F[:, 0] != F[:, 2])]
    return np.ascontiguousarray(V.view(pts.dtype).reshape(-1, 3)), F


def write_obj(filename: str, V: np.ndarray, F: np.ndarray) -> None:
    """igl::writeOBJ's subset: ``v x y z`` lines (17 significant digits, enough to read
    the doubles back exactly), then 1-based ``f a b c`` lines."""
    with open(filename, "w") as f:
        np.savetxt(f, V, fmt="v %.17g %.17g %.17g")
        np.savetxt(f, F + 1, fmt="f %d %d %d")


class MeshBuilder:
    """MeshBuilder(params, flags, grid_size) (include/mesh_builder.h:19-34)."""

    def __init__(self, grid_side: int = MESH_GRID, particle_radius: int = MESH_PARTICLE_RADIUS,
                 laplacian_smooth: bool = False):
        self.grid_side = int(grid_side)
        self.particle_radius = int(particle_radius)
        self.laplacian_smooth = bool(laplacian_smooth)

    def mesh(self, sim):
        """(V float64, F int32) of the particles' surface, smoothed when laplacian_smooth
        is set (include/mesh_builder.h:195-199)."""
        V, F = sim.surface_indexed(self.grid_side, self.particle_radius)
        if self.laplacian_smooth and F.shape[0] > 0:
            V = sim.smooth_mesh(V, F)
        return V, F

    def computeMesh(self, filename: str, sim) -> int:
        """Writes the surface of the simulation's active particles; returns the face count."""
        V, F = self.mesh(sim)
        write_obj(filename, V, F)
        return int(F.shape[0])
