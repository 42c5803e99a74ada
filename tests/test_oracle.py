"""CPU tests of the oracle: pinned against the reference's own test vectors and
SVD outputs (tests/golden), FP32 vs FP64 agreement, and known-answer substeps."""
import json
import os

import numpy as np
import pytest

from helpers import compare_states

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _linalg():
    with open(os.path.join(GOLDEN, "ref_linalg.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_polar_reference_matrices(oracle_lib, dtype):
    """tests/test_linalg.cu:25-75 — sum |RS - M| < 1e-5, ||RR^T - I||_1 < 1e-5, ||S - S^T||_1 < 1e-5."""
    g = _linalg()
    tol = g["tolerances"][0]
    for vals in g["matrices"]:
        M = np.array(vals, dtype=np.float64).reshape(3, 3)
        R, S = oracle_lib.polar(M, dtype)
        R, S = R[0].astype(np.float64), S[0].astype(np.float64)
        assert np.abs(R @ S - M).sum() < tol * (10 if dtype == np.float32 else 1)
        assert np.abs(R @ R.T - np.eye(3)).sum() < tol
        assert np.abs(S - S.T).sum() < tol


def test_polar_reference_tolerance_fp32_basic(oracle_lib):
    """TestDevicePolar.Basic runs the FP32 device SVD on the first matrix with the 1e-5 bound."""
    g = _linalg()
    M = np.array(g["matrices"][0], np.float32).reshape(3, 3)
    R, S = oracle_lib.polar(M, np.float32)
    assert np.abs(R[0].astype(np.float64) @ S[0] - M).sum() < 1e-5


def test_determinant_identity(oracle_lib):
    """tests/test_linalg.cu:77-91: det(I) == 1 exactly."""
    assert oracle_lib.det_f32(np.eye(3)) == 1.0


def test_svd_matches_reference_svd3(oracle_lib):
    """The oracle's FP32 McAdams SVD against the reference's own svd3_cuda.h outputs."""
    d = np.load(os.path.join(GOLDEN, "ref_svd.npz"))
    A = d["A"]
    U, s, V = oracle_lib.svd(A, np.float32)
    # singular values and the polar rotation U V^T agree to FP32 rounding
    assert np.abs(s - d["s"]).max() < 2e-5 * max(1.0, float(np.abs(d["s"]).max()))
    R_ref = np.einsum("nij,nkj->nik", d["U"], d["V"])
    R = np.einsum("nij,nkj->nik", U, V)
    near_identity = slice(96, 224)
    assert np.abs(R[near_identity] - R_ref[near_identity]).max() < 5e-6
    # reconstruction quality of both is the same
    rec = np.einsum("nij,nj,nkj->nik", U.astype(np.float64), s, V)
    rec_ref = np.einsum("nij,nj,nkj->nik", d["U"].astype(np.float64), d["s"], d["V"])
    e, e_ref = np.abs(rec - A).max((1, 2)), np.abs(rec_ref - A).max((1, 2))
    assert np.all(e <= np.maximum(2 * e_ref, 1e-5))


def test_svd_fp64_exact(oracle_lib):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((500, 3, 3))
    U, s, V = oracle_lib.svd(A, np.float64)
    rec = np.einsum("nij,nj,nkj->nik", U, s, V)
    assert np.abs(rec - A).max() < 1e-12
    assert np.allclose(np.linalg.det(U), 1) and np.allclose(np.linalg.det(V), 1)
    assert np.allclose(np.abs(s), np.linalg.svd(A, compute_uv=False), atol=1e-12)
    assert np.all(s[:, 0] >= s[:, 1]) and np.all(s[:, 1] >= np.abs(s[:, 2]) - 1e-12)


def _cfg_small(kind):
    from mpm_gb300 import scenes

    if kind == "elastic":
        return scenes.config_elastic(n=3000, seed=2)
    if kind == "liquid":
        return scenes.config_liquid(n=20000, seed=2, N=32)
    if kind == "snow":
        return scenes.config_snow(n=20000, seed=2, N=32)
    return scenes.mixed_scene(n=6000, seed=2)


@pytest.mark.parametrize("kind", ["elastic", "liquid", "snow", "mixed"])
def test_oracle_fp32_vs_fp64(oracle_lib, kind):
    cfg = _cfg_small(kind)
    mats = [m.derived() for m in cfg["materials"]]
    a, ga, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, 3, np.float32, want_grids=True)
    b, gb, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, 3, np.float64, want_grids=True)
    errs = compare_states(a, b, cfg["params"], b)
    assert max(errs.values()) < 1e-5, errs
    assert np.linalg.norm(ga - gb) / np.linalg.norm(gb) < 1e-5


def _single(x, v=(0, 0, 0), N=16, C=None):
    from mpm_gb300 import materials as M

    st = {"x": np.array([x], np.float32), "v": np.array([v], np.float32),
          "C": np.zeros((1, 3, 3), np.float32) if C is None else np.array([C], np.float32),
          "F": np.eye(3, dtype=np.float32)[None].copy(), "Jp": np.ones(1, np.float32),
          "mat": np.zeros(1, np.uint8)}
    params = {"dt": 1e-4, "N": N, "gravity": -9.8, "boundary_mode": 0}
    return st, params, [M.elastic(1e-5).derived()]


def test_known_answer_rest_particle_falls(oracle_lib):
    """A particle at rest with F = I feels no stress: one substep gives v = dt g e_y."""
    st, p, mats = _single((0.5, 0.5, 0.5))
    out, g, gop = oracle_lib.substep(st, p, mats, 1, np.float64, want_grids=True)
    assert np.allclose(out["v"][0], [0, np.float32(1e-4) * np.float32(-9.8), 0], rtol=1e-6, atol=1e-15)
    assert np.allclose(out["x"][0], st["x"][0] + 1e-4 * out["v"][0], atol=1e-12)
    assert abs(g[..., 3].sum() - mats[0]["particle_mass"]) < 1e-12 * mats[0]["particle_mass"] + 1e-18
    assert np.abs(out["C"]).max() < 1e-9


def test_known_answer_uniform_translation(oracle_lib):
    """Uniform velocity away from walls (gravity off): v preserved, C = 0."""
    rng = np.random.default_rng(0)
    n = 2000
    from mpm_gb300 import materials as M

    st = {"x": (0.4 + 0.2 * rng.random((n, 3))).astype(np.float32),
          "v": np.tile(np.array([0.3, -0.2, 0.1], np.float32), (n, 1)),
          "C": np.zeros((n, 3, 3), np.float32), "F": np.tile(np.eye(3, dtype=np.float32), (n, 1, 1)),
          "Jp": np.ones(n, np.float32), "mat": np.zeros(n, np.uint8)}
    p = {"dt": 1e-4, "N": 32, "gravity": 0.0, "boundary_mode": 0}
    out, _, _ = oracle_lib.substep(st, p, [M.elastic(1e-6).derived()], 1, np.float64)
    assert np.allclose(out["v"], st["v"], atol=1e-12)
    assert np.abs(out["C"]).max() < 1e-9


def test_known_answer_rigid_rotation(oracle_lib):
    """Rigid rotation v = w x (x - c) with matching APIC C (skew matrix): C stays the
    skew matrix of w and the angular velocity is preserved."""
    rng = np.random.default_rng(1)
    n = 4000
    from mpm_gb300 import materials as M

    c = np.array([0.5, 0.5, 0.5])
    w = np.array([0.0, 0.0, 2.0])
    x = c + (rng.random((n, 3)) - 0.5) * 0.2
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    v = (x - c) @ W.T
    st = {"x": x.astype(np.float32), "v": v.astype(np.float32),
          "C": np.tile(W, (n, 1, 1)).astype(np.float32), "F": np.tile(np.eye(3), (n, 1, 1)).astype(np.float32),
          "Jp": np.ones(n, np.float32), "mat": np.zeros(n, np.uint8)}
    p = {"dt": 1e-4, "N": 32, "gravity": 0.0, "boundary_mode": 0}
    out, _, _ = oracle_lib.substep(st, p, [M.elastic(1e-6, E=1.0).derived()], 1, np.float64)
    assert np.abs(out["C"] - W).max() < 1e-6
    assert np.abs(out["v"] - (out["x"] - c) @ W.T).max() < 1e-4


def test_known_answer_snow_clamp(oracle_lib):
    """MMSnow::endOfStepMutation on F = diag(1.1, 1, 0.9): singular values clamped to
    [0.975, 1.0075], Jp *= det(F_old) / det(F_new)."""
    from mpm_gb300 import materials as M

    st, p, _ = _single((0.5, 0.5, 0.5))
    st["F"][0] = np.diag([1.1, 1.0, 0.9])
    p["gravity"] = 0.0
    mats = [M.snow(1e-5).derived()]
    out, _, _ = oracle_lib.substep(st, p, mats, 1, np.float64)
    # trial F of the substep, then the clamp applied by hand
    Ftr = (np.eye(3) + 1e-4 * out["C"][0]) @ st["F"][0].astype(np.float64)
    U, sv_tr, Vt = np.linalg.svd(Ftr)
    sv_cl = np.clip(sv_tr, mats[0]["clamp_lo"], mats[0]["clamp_hi"])
    assert np.abs(out["F"][0] - U @ np.diag(sv_cl) @ Vt).max() < 1e-9
    sv = np.linalg.svd(out["F"][0], compute_uv=False)
    assert np.allclose(sv, [np.float32(1.0075), 1.0, np.float32(0.975)], atol=1e-4)
    expect = np.clip(np.linalg.det(Ftr) / np.prod(sv_cl), 0.6, 20)
    assert abs(out["Jp"][0] - expect) < 1e-9


def test_mass_conservation_p2g(oracle_lib):
    """Grid mass after P2G equals the particle mass (partition of unity) away from walls."""
    from mpm_gb300 import scenes

    cfg = scenes.config_elastic(n=5000, seed=4)
    mats = [m.derived() for m in cfg["materials"]]
    _, g, gop = oracle_lib.substep(cfg["state"], cfg["params"], mats, 1, np.float64, want_grids=True)
    total = 5000 * float(mats[0]["particle_mass"])
    assert abs(g[..., 3].sum() - total) < 1e-10 * total
    # reference quirk: the grid op divides the mass slot by itself (src/mpm.cu:86-88)
    occupied = g[..., 3] > 0
    assert np.all(gop[..., 3][occupied] == 1.0)


def test_g2p_guard_freezes_high_indices(oracle_lib):
    """src/mpm.cu:114: with the guard only particles 0..N^3 run G2P."""
    from mpm_gb300 import scenes

    cfg = scenes.config_elastic(n=5000, seed=5, N=8)
    p = dict(cfg["params"], g2p_guard=1)
    mats = [m.derived() for m in cfg["materials"]]
    out, _, _ = oracle_lib.substep(cfg["state"], p, mats, 1, np.float64)
    lim = 8 ** 3
    assert np.array_equal(out["x"][lim + 1:], cfg["state"]["x"][lim + 1:].astype(np.float64))
    assert not np.array_equal(out["x"][:lim + 1], cfg["state"]["x"][:lim + 1].astype(np.float64))


def _golden_ids():
    from helpers import golden_substep_cases

    return [c[0] for c in golden_substep_cases()]


@pytest.mark.parametrize("case", _golden_ids())
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_substep_matches_reference_policies(oracle_lib, case, dtype):
    """The oracle against the reference's own TransferScheme / MaterialModel (MMSnow) /
    InterpolationKernel / linalg code, compiled for the host (tests/golden/ref_substep.npz):
    every particle field and the grid after P2G within 1e-5 relative after 1-4 substeps."""
    from helpers import golden_substep_cases

    name, cfg, nsteps, expect, grid = next(c for c in golden_substep_cases() if c[0] == case)
    mats = [m.derived() for m in cfg["materials"]]
    out, g_p2g, _ = oracle_lib.substep(cfg["state"], cfg["params"], mats, nsteps, dtype, want_grids=True)
    errs = compare_states(out, expect, cfg["params"], cfg["state"])
    assert max(errs.values()) < 1e-5, errs
    assert np.linalg.norm(g_p2g - grid) < 1e-5 * np.linalg.norm(grid)
