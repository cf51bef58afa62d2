"""The 2-D (triangle mesh) oracle: polar_svd<2> with the 2-D dsvd
(src/variables/mixed_stretch.cpp:43-78, src/svd/dsvd.cpp:140-189), the
3-vector materials (the Vector3d sections of src/energies/*.cpp), and the
Newton timestep of Tri2DMesh + MixedStretch<2>.

The reference holds no 2-D test, so these pin the restatement by finite
differences, by the reference's generated energy expressions written out
again here, and by conservation laws of the whole step.
"""
import os

import numpy as np
import pytest

import oracle
from mfem_gb300 import abi
from mfem_gb300.desc import Tri2dSpec
from mfem_gb300.meshgen import enu_to_lame, square_grid


def _F(rng, scale=0.3):
    return np.eye(2) + scale * rng.uniform(-1, 1, (2, 2))


def test_svd2_sign_fixed_factors():
    rng = np.random.default_rng(1)
    for k in range(50):
        F = rng.uniform(-1, 1, (2, 2))
        sig, U, V = oracle.svd2(F)
        assert np.allclose(U @ np.diag(sig) @ V.T, F, atol=1e-14)
        assert np.isclose(np.linalg.det(U), 1) and np.isclose(np.linalg.det(V), 1)
        assert sig[0] >= abs(sig[1]) - 1e-15
        assert np.sign(sig[1]) == np.sign(np.linalg.det(F))
        assert np.allclose(np.abs(sig), np.linalg.svd(F)[1], atol=1e-14)


def _vec(M):
    return M.ravel(order="F")


def test_polar2_rotation_and_derivative_by_central_differences():
    rng = np.random.default_rng(2)
    for _ in range(20):
        F = _F(rng)
        R, s, dsdF, st = oracle.polar2(F)
        assert st == abi.OK
        assert np.allclose(R.T @ R, np.eye(2), atol=1e-14) and np.isclose(np.linalg.det(R), 1)
        S = R.T @ F
        assert np.isclose(S[0, 1], S[1, 0], atol=1e-14)
        assert np.allclose(s, [S[0, 0], S[1, 1], 0.5 * (S[0, 1] + S[1, 0])])
        sig = np.linalg.svd(F)[1]
        if abs(sig[0] ** 2 - sig[1] ** 2) < 1e-2:
            continue
        h = 1e-6
        fd = np.zeros((3, 4))
        for c in range(4):
            d = np.zeros(4)
            d[c] = h
            sp = oracle.polar2((_vec(F) + d).reshape(2, 2, order="F"), False)[1]
            sm = oracle.polar2((_vec(F) - d).reshape(2, 2, order="F"), False)[1]
            fd[:, c] = (sp - sm) / (2 * h)
        assert np.abs(fd - dsdF).max() < 1e-8


def test_polar2_near_equal_singular_values_drop_the_rotation_term():
    """dsvd sets 1/(s1^2 - s0^2) to 0 below 1e-4 (dsvd.cpp:153-163), so at
    a pure rotation (s0 = s1 = 1) dR/dF = 0 and J = I (x) R^T."""
    th = 0.37
    Rt = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    R, s, dsdF, st = oracle.polar2(Rt)
    assert np.allclose(R, Rt, atol=1e-15) and np.allclose(s, [1, 1, 0], atol=1e-15)
    J = np.kron(np.eye(2), R.T)
    want = np.stack([J[0], J[3], 0.5 * (J[1] + J[2])])
    assert np.allclose(dsdF, want, atol=1e-15)


def device_closed_form_dsdF(F):
    """The closed form the device kernel evaluates: with P = R^T E_rc,
    a = (P01 - P10)/(s0 + s1) (0 where |s0^2 - s1^2| < 1e-4) and
    K = [[0, 1], [-1, 0]], dS/dF_rc = P - a K S."""
    e, f = 0.5 * (F[0, 0] + F[1, 1]), 0.5 * (F[0, 0] - F[1, 1])
    g, h = 0.5 * (F[1, 0] + F[0, 1]), 0.5 * (F[1, 0] - F[0, 1])
    q, r = np.hypot(e, h), np.hypot(f, g)
    R = np.array([[e, -h], [h, e]]) / q
    S = R.T @ F
    K = np.array([[0.0, 1.0], [-1.0, 0.0]])
    out = np.zeros((3, 4))
    small = abs(4 * q * r) < 1e-4
    for c in range(2):
        for rr in range(2):
            E = np.zeros((2, 2))
            E[rr, c] = 1
            P = R.T @ E
            a = 0.0 if small else (P[0, 1] - P[1, 0]) / (2 * q)
            dS = P - a * K @ S
            out[:, rr + 2 * c] = [dS[0, 0], dS[1, 1], 0.5 * (dS[0, 1] + dS[1, 0])]
    return R, out


def test_device_closed_form_equals_the_dsvd_route():
    rng = np.random.default_rng(4)
    for k in range(40):
        F = _F(rng, 0.6) if k % 2 else rng.uniform(-1, 1, (2, 2))
        R, s, dsdF, st = oracle.polar2(F)
        if st != abi.OK:
            continue
        Rc, dc = device_closed_form_dsdF(F)
        assert np.allclose(Rc, R, atol=1e-13)
        assert np.allclose(dc, dsdF, atol=1e-10)


def _ref_energy(mtype, mu, la, s):
    """The reference's generated 3-vector energies, written out again."""
    S1, S2, S3 = s
    if mtype == abi.MATERIAL_SNH:   # stable_neohookean.cpp:236-243
        return (la * (-S1 * S2 + S3 * S3 + 1.0) ** 2) / 2.0 + \
            (mu * (S1 * S1 + S2 * S2 + (S3 * S3) * 2.0 - 2.0)) / 2.0 + mu * (-S1 * S2 + S3 * S3 + 1.0)
    if mtype == abi.MATERIAL_ARAP:  # arap.cpp:67-73
        return (mu * ((S1 - 1.0) ** 2 + (S2 - 1.0) ** 2 + (S3 * S3) * 2.0)) / 2.0
    if mtype == abi.MATERIAL_COROT:  # corotational.cpp:62-69
        return (la * (S1 + S2 - 2.0) ** 2) / 2.0 + mu * ((S1 - 1.0) ** 2 + (S2 - 1.0) ** 2 + (S3 * S3) * 2.0)
    if mtype == abi.MATERIAL_FCR:  # fixed_corotational.cpp:93-100
        return (la * (-S1 * S2 + S3 * S3 + 1.0) ** 2) / 2.0 + \
            mu * ((S1 - 1.0) ** 2 + (S2 - 1.0) ** 2 + (S3 * S3) * 2.0)
    raise ValueError(mtype)


MATS2 = [abi.MATERIAL_SNH, abi.MATERIAL_COROT, abi.MATERIAL_FCR, abi.MATERIAL_ARAP]


@pytest.mark.parametrize("mtype", MATS2)
def test_material2_energy_gradient_hessian(mtype):
    rng = np.random.default_rng(5 + mtype)
    mu, la = 3.0, 7.0
    for _ in range(10):
        s = np.array([1, 1, 0]) + 0.3 * rng.uniform(-1, 1, 3)
        psi, g, H = oracle.material2(mtype, mu, la, s, psd_fix=False)
        assert abs(psi - _ref_energy(mtype, mu, la, s)) < 1e-12
        h = 1e-6
        for k in range(3):
            d = np.zeros(3)
            d[k] = h
            fp, gp, _ = oracle.material2(mtype, mu, la, s + d, psd_fix=False)
            fm, gm, _ = oracle.material2(mtype, mu, la, s - d, psd_fix=False)
            assert abs((fp - fm) / (2 * h) - g[k]) < 1e-7
            assert np.abs((gp - gm) / (2 * h) - H[:, k]).max() < 1e-6
        assert np.allclose(H, H.T)


def test_snh2_hessian_is_psd_projected():
    mu, la = 1.0, 10.0
    s = np.array([0.3, 1.4, 0.8])  # det S < 0: indefinite before the fix
    _, _, H0 = oracle.material2(abi.MATERIAL_SNH, mu, la, s, psd_fix=False)
    _, _, H1 = oracle.material2(abi.MATERIAL_SNH, mu, la, s, psd_fix=True)
    assert np.linalg.eigvalsh(H0).min() < 0
    assert np.linalg.eigvalsh(H1).min() >= 1e-6 - 1e-12 * np.abs(H1).max()
    # the fix keeps the eigenvectors: H1 - H0 is psd
    assert np.linalg.eigvalsh(H1 - H0).min() > -1e-9


def tri2d_spec(nx=8, ny=3, spacing=0.1, E=1e5, nu=0.45, **kw):
    V, T = square_grid(nx, ny, spacing)
    lam, mu = enu_to_lame(E, nu)
    args = dict(V_rest=V, tris=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                density_const=1000.0, bc_type=abi.BC_HANGENDS, bc_ratio=0.01, bc_axis=0,
                dt=0.0333, max_newton_iterations=10, iterative_solver_tolerance=1e-10)
    args.update(kw)
    return Tri2dSpec(**args)


def test_refusals():
    V, T = square_grid(2, 2, 0.1)
    for kw, want in [(dict(material=np.full(len(T), abi.MATERIAL_NH)), abi.ERR_UNSUPPORTED),
                     (dict(material=np.full(len(T), abi.MATERIAL_FUNG)), abi.ERR_UNSUPPORTED),
                     (dict(linear_solver=abi.SOLVER_MINRES_ID), abi.ERR_UNSUPPORTED),
                     (dict(tris=T[:, [0, 2, 1]]), abi.ERR_INVALID),
                     (dict(bdf_order=7), abi.ERR_INVALID)]:
        spec = tri2d_spec(2, 2, **kw)
        with pytest.raises(RuntimeError, match=f"status {want}"):
            oracle.OracleTri2d(spec)


def test_mass_and_system_structure():
    spec = tri2d_spec(5, 3)
    sc = oracle.OracleTri2d(spec)
    rp, col, val, rhs = sc.get_system()
    n = sc.n_free
    A = np.zeros((2 * n, 2 * n))
    for r in range(n):
        for q in range(rp[r], rp[r + 1]):
            A[2 * r:2 * r + 2, 2 * col[q]:2 * col[q] + 2] = val[q]
    assert np.allclose(A, A.T, rtol=0, atol=1e-9 * np.abs(A).max())
    assert np.linalg.eigvalsh(A).min() > 0
    # at rest with gravity the RHS is the gravity load h^2 M g on free rows
    # (elastic terms vanish at S = I): y components all negative, x ~ 0
    assert np.abs(rhs[0::2]).max() < 1e-12 * np.abs(rhs).max()
    assert (rhs[1::2] < 0).all()


def test_free_body_conserves_momentum():
    """No pins, no gravity, a stretched initial state: the internal forces
    of every triangle sum to zero (its dphi/dX rows do), so the linear
    momentum sum_ab M_ab v_b = sum_b m_b v_b (m the row sums of M) stays
    zero while the body oscillates.  (Backward Euler does not conserve
    angular momentum, so that is not checked.)"""
    V, T = square_grid(6, 3, 0.1)
    Vi = V * np.array([1.2, 0.9]) + np.array([0.0, 0.05]) * V[:, :1]
    spec = tri2d_spec(6, 3, bc_type=abi.BC_NULL, body_force=(0.0, 0.0), V_init=Vi,
                      E=1e4, max_newton_iterations=20)
    sc = oracle.OracleTri2d(spec)
    V0, T0 = spec.V_rest, spec.tris
    X = V0[T0]
    area2 = (X[:, 1, 0] - X[:, 0, 0]) * (X[:, 2, 1] - X[:, 0, 1]) - \
        (X[:, 2, 0] - X[:, 0, 0]) * (X[:, 1, 1] - X[:, 0, 1])
    m = np.zeros(len(V0))
    for k in range(3):
        np.add.at(m, T0[:, k], 1000.0 * area2 / 3)   # row sums of rho vol/12 (1 + delta)
    for _ in range(5):
        st = sc.step()
        assert st.status in (abi.OK, abi.ERR_CG_MAXITER)
        s = sc.get_state()
        p = (m[:, None] * s["v"]).sum(0)
        scale = (m[:, None] * np.abs(s["v"])).sum()
        assert scale > 0
        assert np.abs(p).max() < 1e-7 * scale


def test_hanging_sheet_sags_and_converges():
    spec = tri2d_spec(10, 2, newton_residual_tolerance=0.0)
    sc = oracle.OracleTri2d(spec)
    y0 = sc.get_state()["x"][:, 1].copy()
    for _ in range(4):
        st = sc.step()
        assert st.status == abi.OK
        assert st.residual < 1e-6 * st.residual0
    x = sc.get_state()["x"]
    assert np.isfinite(x).all() and x[:, 1].min() < y0.min()


@pytest.mark.parametrize("bc", [abi.BC_STRETCH, abi.BC_TWIST, abi.BC_BEND, abi.BC_SCALEF,
                                abi.BC_ONEPOINT, abi.BC_HANG, abi.BC_PINMIN, abi.BC_COMPRESS])
def test_bc_scripts_step(bc):
    spec = tri2d_spec(6, 2, bc_type=bc, bc_ratio=0.1, bc_velocity=0.2,
                      max_newton_iterations=4)
    sc = oracle.OracleTri2d(spec)
    for _ in range(3):
        st = sc.step()
        assert st.status in (abi.OK, abi.ERR_CG_MAXITER, abi.ERR_LS_FAILED)
    assert np.isfinite(sc.get_state()["x"]).all()


def test_results_do_not_depend_on_the_thread_count():
    """Element loops run in parallel; every sum is a fixed-order chunked sum."""
    out = []
    for threads in (1, 4):
        oracle.set_threads(threads)
        sc = oracle.OracleTri2d(tri2d_spec(40, 10))
        for _ in range(2):
            sc.step()
        out.append(sc.get_state())
    oracle.set_threads(os.cpu_count())
    for k in ("x", "v", "s", "R"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_newton_direction_solves_the_linearised_kkt_system():
    """The direction that the Schur system and the local solve produce
    satisfies the linearised KKT conditions of the mixed problem, checked
    with D = ds/dF from central differences of polar_svd<2>'s s (not the
    dsvd route), B = Jloc from dphi/dX, the material's H = h^2 hess psi and
    g = h^2 grad psi, and the P1 mass written out again here:
      M (x + dx - x~ - h^2 f) - sum_e vol_e B_e^T D_e^T Sym la_e = 0  (free rows)
      Sym la_e + H_e ds_e + g_e = 0
      ds_e = S_e(x) - s_e + D_e B_e dx_e."""
    rng = np.random.default_rng(21)
    V0, T = square_grid(6, 3, 0.1)
    Vi = V0 + 0.015 * rng.uniform(-1, 1, V0.shape)
    sp = tri2d_spec(6, 3, V_init=Vi, iterative_solver_tolerance=1e-13,
                    max_iterative_solver_iters=20000)
    sc = oracle.OracleTri2d(sp)
    sc.step()                      # so that s differs from S(x) and v from 0
    st = sc.get_state()
    x, v, s = st["x"], st["v"], st["s"]
    h = sp.dt
    xt = x + h * v                 # BDF1: x~ = x + h v
    dx, ds, la, _ = sc.direction()
    sym = np.array([1.0, 1.0, 2.0])
    nv, nt = len(V0), len(T)
    M = np.zeros((nv, nv))
    rhsA = np.zeros((nv, 2))
    lam, mu = sp.lam[0], sp.mu[0]
    f = np.array([0.0, float(np.float32(-9.8))])
    worst_b = worst_c = 0.0
    for e in range(nt):
        X = V0[T[e]]
        Dm = np.stack([X[1] - X[0], X[2] - X[0]], axis=1)
        vol = np.linalg.det(Dm)
        Di = np.linalg.inv(Dm)
        dX = np.vstack([-Di.sum(axis=0), Di[0], Di[1]])        # dphi_k/dX_c
        for a in range(3):
            for b in range(3):
                M[T[e, a], T[e, b]] += 1000.0 * vol / 12 * (2 if a == b else 1)
        B = np.zeros((4, 6))
        for k in range(3):
            for c in range(2):
                for r in range(2):
                    B[r + 2 * c, 2 * k + r] = dX[k, c]
        xe = x[T[e]].ravel()
        Fv = B @ xe
        D = np.zeros((3, 4))
        eps = 1e-7
        for c in range(4):
            d = np.zeros(4)
            d[c] = eps
            sp_ = oracle.polar2((Fv + d).reshape(2, 2, order="F"), False)[1]
            sm_ = oracle.polar2((Fv - d).reshape(2, 2, order="F"), False)[1]
            D[:, c] = (sp_ - sm_) / (2 * eps)
        S = oracle.polar2(Fv.reshape(2, 2, order="F"), False)[1]
        _, g, H = oracle.material2(abi.MATERIAL_SNH, mu, lam, s[e])
        g, H = h * h * g, h * h * H
        rb = sym * la[e] + H @ ds[e] + g
        worst_b = max(worst_b, np.abs(rb).max() / (np.abs(g).max() + np.abs(H @ ds[e]).max()))
        rc = ds[e] - (S - s[e] + D @ B @ dx[T[e]].ravel())
        worst_c = max(worst_c, np.abs(rc).max() / max(np.abs(ds[e]).max(), 1e-12))
        rhsA[T[e]] -= vol * (B.T @ D.T @ (sym * la[e])).reshape(3, 2)
    assert worst_b < 1e-9
    assert worst_c < 1e-6
    ra = M @ (x + dx - xt - h * h * f) + rhsA
    free = V0[:, 0] <= V0[:, 0].max() - 0.01 * np.ptp(V0[:, 0])
    scale = np.abs(M @ (x - xt - h * h * f)).max()
    assert np.abs(ra[free]).max() < 1e-6 * scale


def test_tri2d_golden_regression():
    """The 2-D oracle against its committed fixture
    (tests/golden/make_golden.py: write_tri2d)."""
    import sys
    gold_dir = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, gold_dir)
    try:
        import make_golden
    finally:
        sys.path.remove(gold_dir)
    gold = np.load(os.path.join(gold_dir, "tri2d_oracle_fp64.npz"))
    sc = oracle.OracleTri2d(make_golden.tri2d_sheet_spec())
    for step in range(1, 11):
        sc.step()
        if step in (1, 10):
            assert np.allclose(sc.get_state()["x"], gold[f"x_{step}"], atol=1e-10, rtol=0)
