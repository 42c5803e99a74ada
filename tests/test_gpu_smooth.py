"""GPU tests of the Laplacian smoothing (mpm_surface_smooth / mpm_surface_smooth_device,
MeshBuilder::smoothMesh of include/mesh_builder.h:212-245) against the oracle's direct
sparse solve of the same system (oracle/smooth_oracle.py).

The GPU solves (M - 0.001 L) U = M V by preconditioned conjugate gradients to a relative
residual of 1e-12 per coordinate; the bar is |U_gpu - U_oracle| <= 1e-9 max|U_oracle|,
which leaves a factor of 1000 for the system's condition number.  Inputs: the meshes the
reference's own MeshBuilder::computeMesh wrote for seeded particles (tests/golden), a
sphere, an open mesh with unused vertices, and a simulated body's surface."""
import ctypes

import numpy as np
import pytest

from helpers import icosphere, open_icosphere
from surface_checks import golden_meshes

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _sim(x=None, N=32):
    from mpm_gb300 import materials as M
    from mpm_gb300.simulation import Simulation

    sim = Simulation(dt=1e-4, N=N, sort_interval=4)
    if x is None:
        x = np.full((8, 3), 0.5, np.float32)
    sim.set_materials([M.elastic(1.0 / len(x))])
    sim.upload({"x": x})
    return sim


def _oracle():
    pytest.importorskip("scipy")
    from oracle import smooth_oracle

    return smooth_oracle


def _check(U, ref):
    err = np.abs(U - ref).max()
    assert err <= TOL * np.abs(ref).max(), (err, np.abs(ref).max())


GOLDEN = [m for m in golden_meshes() if m[5] is not None]


@pytest.mark.parametrize("case", GOLDEN, ids=[m[0] for m in GOLDEN])
def test_smooth_reference_meshes(gpu_lib, case):
    so = _oracle()
    name, _, _, _, _, V, F, _, _, _ = case
    sim = _sim()
    U = sim.smooth_mesh(V, F)
    _check(U, so.smooth_mesh(V, F))
    np.testing.assert_allclose(0.5 * so.doublearea(U, F).sum(), 1.0, rtol=1e-12)
    assert 0 < sim.smooth_iterations < 20000


def test_smooth_is_reproducible(gpu_lib):
    """Every sum of the solver runs in a fixed order: two calls agree bit for bit."""
    V, F = GOLDEN[0][5], GOLDEN[0][6]
    sim = _sim()
    a = sim.smooth_mesh(V, F)
    b = sim.smooth_mesh(V, F)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_smooth_sphere_and_open_mesh(gpu_lib):
    so = _oracle()
    sim = _sim()
    V, F = icosphere(4)
    _check(sim.smooth_mesh(V, F), so.smooth_mesh(V, F))
    # an open mesh whose cap vertices no face uses any more: those keep their positions
    V, F = open_icosphere(3)
    V = V.astype(np.float64) * 2.5 + 0.3
    U = sim.smooth_mesh(V, F)
    _check(U, so.smooth_mesh(V, F))
    unused = np.setdiff1d(np.arange(len(V)), F)
    assert len(unused) > 0
    ratio = U[unused] / V[unused]
    np.testing.assert_allclose(ratio, ratio[0, 0], rtol=1e-12)


def test_smooth_simulated_surface(gpu_lib):
    """The surface of a settled body (mpm_surface_mesh_indexed), smoothed, through the
    MeshBuilder option the reference's --laplacian_smooth maps to."""
    so = _oracle()
    from mpm_gb300.mesh_builder import MeshBuilder

    rng = np.random.default_rng(11)
    u = rng.normal(size=(30000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    x = (0.5 + 0.18 * u * rng.random(30000)[:, None] ** (1 / 3)).astype(np.float32)
    sim = _sim(x, 32)
    sim.advance(20)
    V, F = sim.surface_indexed(96, 3)
    assert len(F) > 5000
    U, F2 = MeshBuilder(96, 3, laplacian_smooth=True).mesh(sim)
    assert np.array_equal(F2, F)
    _check(U, so.smooth_mesh(V, F))


def test_smooth_device_matches_host(gpu_lib):
    torch = pytest.importorskip("torch")
    from mpm_gb300 import _lib

    sim = _sim()
    V, F = icosphere(3)
    V = V.astype(np.float64)
    U = sim.smooth_mesh(V, F)
    Vd = torch.from_numpy(V.copy()).cuda()
    Fd = torch.from_numpy(F.astype(np.int32)).cuda()
    torch.cuda.synchronize()
    it = ctypes.c_int32()
    _lib.check(sim.L.mpm_surface_smooth_device(sim.ctx, ctypes.c_void_p(Vd.data_ptr()), len(V),
                                               ctypes.c_void_p(Fd.data_ptr()), len(F), ctypes.byref(it)), sim.ctx)
    Ud = Vd.cpu().numpy()
    _check(Ud, U)
    assert it.value > 0


def test_smooth_errors_and_empty(gpu_lib):
    from mpm_gb300 import _lib

    sim = _sim()
    V, F = icosphere(1)
    V = V.astype(np.float64)
    bad = F.copy()
    bad[3, 1] = len(V)
    with pytest.raises(_lib.MpmError):
        sim.smooth_mesh(V, bad)
    bad[3, 1] = -1
    with pytest.raises(_lib.MpmError):
        sim.smooth_mesh(V, bad)
    # a face of zero area: the reference's cotangent weights are not finite
    Vz = np.vstack([V, V[F[0, 0]], V[F[0, 0]]])
    Fz = np.vstack([F, [[len(V), len(V) + 1, F[0, 0]]]]).astype(np.int32)
    with pytest.raises(_lib.MpmError):
        sim.smooth_mesh(Vz, Fz)
    # vertices without faces: singular
    with pytest.raises(_lib.MpmError):
        sim.smooth_mesh(V, np.zeros((0, 3), np.int32))
    # faces without vertices: every index is out of range
    with pytest.raises(_lib.MpmError):
        sim.smooth_mesh(np.zeros((0, 3)), F)
    # nothing to smooth
    assert sim.smooth_mesh(np.zeros((0, 3)), np.zeros((0, 3), np.int32)).shape == (0, 3)
    # the input is unchanged by a refused call, and the context still works
    U = sim.smooth_mesh(V, F)
    assert np.isfinite(U).all()
    sim.advance(2)
