"""The oracle pinned against the reference's own checks and finite differences.

* tests/test_dsvd.cpp:204-238 ("dRdF"): Procrustes dR/dF vs central
  differences on the reference's own random draw (tests/golden/kat_dRdF.json).
* tests/test_dsvd.cpp:74-110 ("dsvd - dR/dF"): SVD dR/dF vs central differences.
* every material's gradient and Hessian vs central differences of the energy,
  the psd projection, the polar derivative ds/dF, and the PCG solution.
"""
import json
import os

import numpy as np
import pytest

import oracle
from mfem_gb300 import abi, configs

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_kat_dRdF_reference_draw():
    k = json.load(open(os.path.join(GOLD, "kat_dRdF.json")))
    F, S, a = np.array(k["F"]), np.array(k["S"]), k["alpha"]
    fd = np.zeros((9, 9))
    for ii in range(3):
        for jj in range(3):
            P = np.zeros((3, 3))
            P[ii, jj] = a
            R0, _, _ = oracle.procrustes(np.eye(3), S, F + P, False)
            R1, _, _ = oracle.procrustes(np.eye(3), S, F - P, False)
            fd[:, ii + 3 * jj] = ((R0 - R1) / (2 * a)).ravel(order="F")
    R, d, it = oracle.procrustes(np.eye(3), S, F, True, k["tol"], k["max_iter"])
    assert np.linalg.norm(fd - d) <= k["bound"]
    assert np.allclose(R.T @ R, np.eye(3), atol=1e-12)


def test_kat_dsvd_fixed_F():
    F = np.array(json.load(open(os.path.join(GOLD, "kat_dsvd.json")))["F"])

    def polar_R(M):
        U, _, Vt = np.linalg.svd(M)
        return U @ Vt

    d = oracle.dsvd_dRdF(F)
    a = 1e-6
    fd = np.zeros((9, 9))
    for ii in range(3):
        for jj in range(3):
            P = np.zeros((3, 3))
            P[ii, jj] = a
            fd[:, ii + 3 * jj] = ((polar_R(F + P) - polar_R(F - P)) / (2 * a)).ravel(order="F")
    assert np.linalg.norm(fd - d) < 1e-6


def _random_F(rng, scale=0.3):
    return np.eye(3) + scale * rng.uniform(-1, 1, (3, 3))


def test_polar_matches_svd_and_derivative_fd():
    rng = np.random.default_rng(3)
    for _ in range(20):
        F = _random_F(rng)
        R, s, dsdF = oracle.polar(F)
        U, _, Vt = np.linalg.svd(F)
        assert np.allclose(R, U @ Vt, atol=1e-6)
        a = 1e-6
        for ii in range(3):
            for jj in range(3):
                P = np.zeros((3, 3))
                P[ii, jj] = a
                _, sp, _ = oracle.polar(F + P, compute_gradients=False)
                _, sm, _ = oracle.polar(F - P, compute_gradients=False)
                fd = (sp - sm) / (2 * a)
                assert np.allclose(fd, dsdF[:, ii + 3 * jj], atol=2e-5)


@pytest.mark.parametrize("mtype", range(6))
def test_material_derivatives_fd(mtype):
    rng = np.random.default_rng(10 + mtype)
    lam, mu = 2.0e5, 1.0e5
    for _ in range(5):
        F = _random_F(rng, 0.1)
        _, s, _ = oracle.polar(F, compute_gradients=False)
        g = oracle.material_gradient(mtype, mu, lam, s)
        H = oracle.material_hessian(mtype, mu, lam, s, psd_fix=False)
        h = 1e-6
        for i in range(6):
            e = np.zeros(6)
            e[i] = h
            fdg = (oracle.material_energy(mtype, mu, lam, s + e) -
                   oracle.material_energy(mtype, mu, lam, s - e)) / (2 * h)
            assert abs(fdg - g[i]) <= 1e-5 * (abs(g[i]) + mu)
            fdH = (oracle.material_gradient(mtype, mu, lam, s + e) -
                   oracle.material_gradient(mtype, mu, lam, s - e)) / (2 * h)
            assert np.allclose(fdH, H[:, i], atol=1e-4 * mu)
        assert np.allclose(H, H.T)


def test_snh_closed_form_energy():
    """psi = mu/2(|S|^2-3) - mu(J-1) + lam/2 (J-1)^2 (scripts/derivs.m:29)."""
    rng = np.random.default_rng(5)
    mu, lam = 3.0, 7.0
    for _ in range(10):
        S = np.eye(3) + 0.2 * rng.uniform(-1, 1, (3, 3))
        S = 0.5 * (S + S.T)
        s = np.array([S[0, 0], S[1, 1], S[2, 2], S[0, 1], S[0, 2], S[1, 2]])
        J = np.linalg.det(S)
        ref = mu / 2 * (np.sum(S * S) - 3) - mu * (J - 1) + lam / 2 * (J - 1) ** 2
        assert abs(oracle.material_energy(abi.MATERIAL_SNH, mu, lam, s) - ref) < 1e-12


def test_psd_fix_projects_negative_eigenvalues():
    rng = np.random.default_rng(7)
    A = rng.normal(size=(6, 6))
    A = A + A.T
    w, V = np.linalg.eigh(A)
    Hf = oracle.psd_fix(A, 1e-6)
    w2 = np.linalg.eigvalsh(Hf)
    assert w2.min() >= 1e-6 * (1 - 1e-9)
    ref = V @ np.diag(np.maximum(w, 1e-6)) @ V.T
    assert np.allclose(Hf, ref, atol=1e-9)
    B = A + (abs(w.min()) + 1.0) * np.eye(6)          # already PD: unchanged
    assert np.array_equal(oracle.psd_fix(B, 1e-6), B)


def test_oracle_pcg_solves_system():
    sc = oracle.OracleScene(configs.beam_c1())
    rp, col, val, rhs = sc.get_system()
    n = len(rp) - 1
    A = np.zeros((3 * n, 3 * n))
    for r in range(n):
        for q in range(rp[r], rp[r + 1]):
            A[3 * r:3 * r + 3, 3 * col[q]:3 * col[q] + 3] = val[q]
    assert np.allclose(A, A.T, rtol=1e-10, atol=1e-12 * abs(A).max())
    assert np.linalg.eigvalsh(A).min() > 0
    x, it, err = sc.pcg(rhs)
    assert err < 1e-8
    assert np.linalg.norm(A @ x - rhs) <= 1.01e-8 * np.linalg.norm(rhs)


def test_oracle_rhs_is_negative_energy_gradient_at_zero_lambda():
    """At the first Newton iteration (lambda = 0) with s = S(x), the Schur
    right-hand side equals -dE/dx of the incremental potential
    E(x) = 1/2|x - x~ - h^2 f|_M^2 + h^2 sum vol psi(S(x))."""
    spec = configs.beam_c1()
    base = oracle.OracleScene(spec)
    x0 = base.get_state()["x"]
    free = np.where(spec.is_fixed == 0)[0]
    rng = np.random.default_rng(2)
    x = x0 + rng.uniform(-0.002, 0.002, x0.shape) * (spec.is_fixed[:, None] == 0)

    def scene_at(xf):
        sc = oracle.OracleScene(spec)     # x~ = x0 (scene at rest)
        sc.set_positions(xf)
        out = sc.elem_update(xf.ravel(), spec.dt)
        sc.set_state(s=out["S"])          # s = S(x): constraint satisfied
        return sc

    _, _, _, rhs = scene_at(x).get_system()
    for k in [0, 5, 17, 40, 88]:
        v, c = free[k // 3], k % 3
        xp, xm = x.copy(), x.copy()
        xp[v, c] += 1e-7
        xm[v, c] -= 1e-7
        fd = (scene_at(xp).energy(0.0) - scene_at(xm).energy(0.0)) / 2e-7
        assert abs(-fd - rhs[k]) <= 1e-5 * np.abs(rhs).max()


def test_oracle_beam_golden_regression():
    gold = np.load(os.path.join(GOLD, "c1_oracle_fp64.npz"))
    sc = oracle.OracleScene(configs.beam_c1())
    for step in range(1, 11):
        sc.step()
        if step in (1, 10):
            assert np.allclose(sc.get_state()["x"], gold[f"x_{step}"], atol=1e-9, rtol=0)
