"""The 3-D Newton direction against the linearised KKT conditions of the
mixed problem, with every ingredient written out again here: the polar
factor by numpy's SVD (not Procrustes), ds/dF by central differences of it,
Jloc from dphi/dX, the P1 mass, and the material's h^2 grad/hess psi.  The
(dx, ds, lambda) of the Schur system + local solve (MixedStretch::solve,
mixed_stretch.cpp:243-259) must satisfy
  M (x + dx - x~ - h^2 f) - sum_e vol_e B_e^T D_e^T Sym la_e = 0  (free rows)
  Sym la_e + H_e ds_e + g_e = 0
  ds_e = S_e(x) - s_e + D_e B_e dx_e
which pins the whole reduction (assembly, RHS, local solve) independently
of the oracle's own derivative code."""
import numpy as np

import oracle
from mfem_gb300 import abi
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask

SYM = np.array([1.0, 1.0, 1.0, 2.0, 2.0, 2.0])


def _svec(F):
    U, _, Vt = np.linalg.svd(F)
    if np.linalg.det(U @ Vt) < 0:
        U[:, -1] = -U[:, -1]
    S = (U @ Vt).T @ F
    return np.array([S[0, 0], S[1, 1], S[2, 2], 0.5 * (S[1, 0] + S[0, 1]),
                     0.5 * (S[2, 0] + S[0, 2]), 0.5 * (S[2, 1] + S[1, 2])])


def test_newton_direction_solves_the_linearised_kkt_system():
    V0, T = cube_grid(4, 2, 2, 0.05)
    lam, mu = enu_to_lame(2e5, 0.4)
    fixed = face_mask(V0, 0, "min")
    spec = SceneSpec(V_rest=V0, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=fixed, dt=1 / 60, max_newton_iterations=2,
                     iterative_solver_tolerance=1e-13, max_iterative_solver_iters=20000,
                     precision=abi.PRECISION_FP64)
    sc = oracle.OracleScene(spec)
    sc.step()                           # s differs from S(x), v from 0
    st = sc.get_state()
    x, v, s = st["x"], st["v"], st["s"]
    h = spec.dt
    xt = x + h * v                      # BDF1
    sc.update_system()
    kkt, _, _ = sc.schur_solve()
    free = np.where(fixed == 0)[0]
    nf, nt, nv = len(free), len(T), len(V0)
    dx = np.zeros((nv, 3))
    dx[free] = kkt[:3 * nf].reshape(-1, 3)
    ds = kkt[3 * nf:3 * nf + 6 * nt].reshape(-1, 6)
    la = kkt[3 * nf + 6 * nt:].reshape(-1, 6)
    f = np.array([0.0, float(np.float32(-9.8)), 0.0])
    M = np.zeros((nv, nv))
    force = np.zeros((nv, 3))
    worst_b = worst_c = 0.0
    for e in range(nt):
        X = V0[T[e]]
        Dm = (X[1:] - X[0]).T
        vol = abs(np.linalg.det(Dm)) / 6
        Di = np.linalg.inv(Dm)
        dX = np.vstack([-Di.sum(axis=0), Di])          # dphi_k/dX_c
        for a in range(4):
            for b in range(4):
                M[T[e, a], T[e, b]] += 1000.0 * vol / 20 * (2 if a == b else 1)
        B = np.zeros((9, 12))
        for k in range(4):
            for c in range(3):
                for r in range(3):
                    B[r + 3 * c, 3 * k + r] = dX[k, c]
        Fv = B @ x[T[e]].ravel()
        D = np.zeros((6, 9))
        eps = 1e-7
        for c in range(9):
            d = np.zeros(9)
            d[c] = eps
            D[:, c] = (_svec((Fv + d).reshape(3, 3, order="F")) -
                       _svec((Fv - d).reshape(3, 3, order="F"))) / (2 * eps)
        S = _svec(Fv.reshape(3, 3, order="F"))
        g = h * h * oracle.material_gradient(abi.MATERIAL_SNH, mu, lam, s[e])
        H = h * h * oracle.material_hessian(abi.MATERIAL_SNH, mu, lam, s[e])
        rb = SYM * la[e] + H @ ds[e] + g
        worst_b = max(worst_b, np.abs(rb).max() / (np.abs(g).max() + np.abs(H @ ds[e]).max()))
        rc = ds[e] - (S - s[e] + D @ B @ dx[T[e]].ravel())
        worst_c = max(worst_c, np.abs(rc).max() / max(np.abs(ds[e]).max(), 1e-12))
        force[T[e]] -= vol * (B.T @ D.T @ (SYM * la[e])).reshape(4, 3)
    assert worst_b < 1e-9
    assert worst_c < 1e-5
    ra = M @ (x + dx - xt - h * h * f) + force
    scale = np.abs(M @ (x - xt - h * h * f)).max()
    assert np.abs(ra[free]).max() < 1e-6 * scale
    # the same with lambda's sign flipped is far off (the check has teeth)
    rflip = M @ (x + dx - xt - h * h * f) - force
    assert np.abs(rflip[free]).max() > 1e-2 * scale


def test_line_search_energy_matches_the_incremental_potential():
    """energy_func(alpha) (newton_optimizer.cpp:34-49) at the direction
    above against the mixed incremental potential written out again:
    1/2 d^T M d + h^2 sum vol psi(s + a ds) - sum vol la^T Sym (S(x + a dx) -
    s - a ds), d = x + a dx - x~ - h^2 f, S from numpy's SVD polar."""
    V0, T = cube_grid(4, 2, 2, 0.05)
    lam, mu = enu_to_lame(2e5, 0.4)
    fixed = face_mask(V0, 0, "min")
    spec = SceneSpec(V_rest=V0, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=fixed, dt=1 / 60, max_newton_iterations=2,
                     iterative_solver_tolerance=1e-13, max_iterative_solver_iters=20000,
                     precision=abi.PRECISION_FP64)
    sc = oracle.OracleScene(spec)
    sc.step()
    st = sc.get_state()
    x, v, s = st["x"], st["v"], st["s"]
    h = spec.dt
    xt = x + h * v
    sc.update_system()
    kkt, _, _ = sc.schur_solve()
    free = np.where(fixed == 0)[0]
    nf, nt, nv = len(free), len(T), len(V0)
    dx = np.zeros((nv, 3))
    dx[free] = kkt[:3 * nf].reshape(-1, 3)
    ds = kkt[3 * nf:3 * nf + 6 * nt].reshape(-1, 6)
    la = kkt[3 * nf + 6 * nt:].reshape(-1, 6)
    f = np.array([0.0, float(np.float32(-9.8)), 0.0])
    M = np.zeros((nv, nv))
    vols, Bs = [], []
    for e in range(nt):
        X = V0[T[e]]
        Dm = (X[1:] - X[0]).T
        vol = abs(np.linalg.det(Dm)) / 6
        Di = np.linalg.inv(Dm)
        dX = np.vstack([-Di.sum(axis=0), Di])
        for a in range(4):
            for b in range(4):
                M[T[e, a], T[e, b]] += 1000.0 * vol / 20 * (2 if a == b else 1)
        B = np.zeros((9, 12))
        for k in range(4):
            for c in range(3):
                for r in range(3):
                    B[r + 3 * c, 3 * k + r] = dX[k, c]
        vols.append(vol)
        Bs.append(B)
    for a in (0.0, 0.25, 1.0):
        xa = x + a * dx
        d = xa - xt - h * h * f
        E = 0.5 * np.sum(d * (M @ d))
        scale = abs(E)
        for e in range(nt):
            sa = s[e] + a * ds[e]
            S = _svec((Bs[e] @ xa[T[e]].ravel()).reshape(3, 3, order="F"))
            ep = h * h * vols[e] * oracle.material_energy(abi.MATERIAL_SNH, mu, lam, sa)
            ec = vols[e] * np.dot(la[e], SYM * (S - sa))
            E += ep - ec
            scale += abs(ep) + abs(ec)
        # against the sizes of the terms; the oracle's S is Procrustes'
        # (converged to its 1e-6 gradient tolerance, about 1e-13 in S here),
        # this one numpy's SVD
        assert abs(sc.energy(a) - E) <= 1e-9 * scale
