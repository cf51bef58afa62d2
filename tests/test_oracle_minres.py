"""The (x, s, lambda) system of "minres-indefinite-block" in the oracle
(SystemMatrixIndefinite, linear_system.h:61-99; BlockMatrix product,
block_matrix.h:63-126) against the reduced path it must agree with."""
import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask


def _spec(solver, tol, iters, dims=(6, 3, 3), E=2e5, newton=3):
    V, T = cube_grid(*dims, 0.05)
    lam, mu = enu_to_lame(E, 0.4)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, 0, "min"), dt=1 / 60, max_newton_iterations=newton,
                     iterative_solver_tolerance=tol, max_iterative_solver_iters=iters,
                     linear_solver=solver, precision=abi.PRECISION_FP64)


@pytest.fixture(scope="module")
def loaded():
    """A beam after one step (deformed, non-zero multipliers), system updated."""
    import oracle
    o = oracle.OracleScene(_spec(abi.SOLVER_EIGEN_CG_DIAG, 1e-13, 5000, newton=2))
    o.step()
    o.update_system()
    return o


def test_kkt_operator_is_symmetric(loaded):
    n = len(loaded.kkt_rhs())
    rng = np.random.default_rng(3)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    a, b = u @ loaded.kkt_mul(v), v @ loaded.kkt_mul(u)
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)


def test_schur_solution_solves_the_full_system(loaded):
    rhs = loaded.kkt_rhs()
    x, it, err = loaded.schur_solve()
    r = loaded.kkt_mul(x) - rhs
    nx = 3 * loaded.n_free
    ns = 6 * loaded.n_tets
    # x and s rows to the PCG tolerance; lambda rows are a constraint whose
    # right-hand side is near zero, compared against the row scale instead
    assert np.linalg.norm(r[:nx]) <= 1e-10 * np.linalg.norm(rhs[:nx])
    assert np.linalg.norm(r[nx:nx + ns]) <= 1e-10 * np.linalg.norm(rhs[:nx])
    assert np.linalg.norm(r[nx + ns:]) <= 1e-10 * np.linalg.norm(rhs[:nx])


def test_minres_solution_matches_the_reduced_path(loaded):
    rhs = loaded.kkt_rhs()
    xs, _, _ = loaded.schur_solve()
    xm, it, err, st = loaded.minres(rhs)
    assert st == abi.OK and err < 1e-13 and 0 < it < 13000
    nx = 3 * loaded.n_free
    assert np.abs(xm[:nx] - xs[:nx]).max() <= 1e-8 * np.abs(xs[:nx]).max()


def test_minres_steps_match_pcg_steps_at_tight_tolerance():
    import oracle
    a = oracle.OracleScene(_spec(abi.SOLVER_EIGEN_CG_DIAG, 1e-13, 5000))
    b = oracle.OracleScene(_spec(abi.SOLVER_MINRES_ID, 1e-13, 20000))
    for _ in range(2):
        sa, sb = a.step(), b.step()
        assert sa.status == abi.OK and sb.status == abi.OK
        assert sa.newton_iterations == sb.newton_iterations
    xa, xb = a.get_state()["x"], b.get_state()["x"]
    V0 = _spec(abi.SOLVER_EIGEN_CG_DIAG, 1e-13, 5000).V_rest
    assert np.abs(xa - xb).max() <= 1e-10 * np.abs(xa - V0).max()


def test_minres_at_the_scene_tolerance_converges_each_newton_iteration():
    import oracle
    b = oracle.OracleScene(_spec(abi.SOLVER_MINRES_ID, 1e-4, 500))
    for _ in range(3):
        st = b.step()
        assert st.status == abi.OK and st.cg_error < 1e-4
