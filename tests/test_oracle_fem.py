"""The standard-FEM "stretch" variable in the oracle: the 9-vector energies
of Stable-Neohookean and Neohookean (stable_neohookean.cpp:97-234,
neohookean.cpp:96-231) and the Newton system of Stretch::update
(src/variables/stretch.cpp:33-60)."""
import numpy as np
import pytest

from mfem_gb300 import abi, configs


def _F(rng):
    return np.eye(3) + 0.25 * rng.uniform(-1, 1, (3, 3))


@pytest.mark.parametrize("mtype", [abi.MATERIAL_SNH, abi.MATERIAL_NH])
def test_energy_form(mtype):
    import oracle
    rng = np.random.default_rng(11)
    mu, lam = 3.0, 7.0
    for _ in range(10):
        F = _F(rng)
        J = np.linalg.det(F)
        base = mu / 2 * (np.sum(F * F) - 3)
        ref = base + (mu * (1 - J) + lam / 2 * (1 - J) ** 2 if mtype == abi.MATERIAL_SNH
                      else lam / 2 * np.log(J) ** 2 - mu * np.log(J))
        assert abs(oracle.material9(mtype, mu, lam, F)[0] - ref) < 1e-12


@pytest.mark.parametrize("mtype", [abi.MATERIAL_SNH, abi.MATERIAL_NH])
def test_gradient_and_hessian_by_central_differences(mtype):
    import oracle
    rng = np.random.default_rng(12)
    mu, lam = 3.0, 7.0
    for _ in range(5):
        F = _F(rng)
        f = F.ravel(order="F")
        _, g, H = oracle.material9(mtype, mu, lam, F, psd_fix=False)
        h = 1e-6
        for k in range(9):
            d = np.zeros(9)
            d[k] = h
            Fp, Fm = (f + d).reshape(3, 3, order="F"), (f - d).reshape(3, 3, order="F")
            pp, gp, _ = oracle.material9(mtype, mu, lam, Fp, psd_fix=False)
            pm, gm, _ = oracle.material9(mtype, mu, lam, Fm, psd_fix=False)
            assert abs((pp - pm) / (2 * h) - g[k]) <= 1e-7 * max(1.0, abs(g[k]))
            assert np.abs((gp - gm) / (2 * h) - H[:, k]).max() <= 1e-6 * max(1.0, np.abs(H).max())
        assert np.allclose(H, H.T, atol=1e-12)


def test_psd_fixed_hessian():
    import oracle
    rng = np.random.default_rng(13)
    for mtype, tol in ((abi.MATERIAL_SNH, 0.0), (abi.MATERIAL_NH, 1e-6)):
        for _ in range(5):
            _, _, H = oracle.material9(mtype, 3.0, 7.0, _F(rng))
            assert np.linalg.eigvalsh(H).min() >= tol - 1e-9


def _fem_spec(**kw):
    s = configs.beam_c1()
    s.formulation = abi.FORMULATION_STRETCH
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_fem_rhs_is_negative_energy_gradient():
    """-dE/dx of E(x) = 1/2|x - x~ - h^2 f|_M^2 + h^2 sum vol psi(F(x)) is the
    right-hand side Stretch::rhs + Displacement::rhs."""
    import oracle
    spec = _fem_spec()
    x0 = oracle.OracleScene(spec).get_state()["x"]
    free = np.where(spec.is_fixed == 0)[0]
    rng = np.random.default_rng(2)
    x = x0 + rng.uniform(-0.002, 0.002, x0.shape) * (spec.is_fixed[:, None] == 0)

    def scene_at(xf):
        sc = oracle.OracleScene(spec)
        sc.set_positions(xf)
        return sc

    _, _, _, rhs = scene_at(x).get_system()
    for k in [0, 5, 17, 40, 88]:
        v, c = free[k // 3], k % 3
        xp, xm = x.copy(), x.copy()
        xp[v, c] += 1e-7
        xm[v, c] -= 1e-7
        fd = (scene_at(xp).energy(0.0) - scene_at(xm).energy(0.0)) / 2e-7
        assert abs(-fd - rhs[k]) <= 1e-5 * np.abs(rhs).max()


def test_fem_steps_converge_and_sag():
    import oracle
    sc = oracle.OracleScene(_fem_spec())
    y0 = sc.get_state()["x"][:, 1].min()
    for _ in range(5):
        st = sc.step()
        assert st.status == abi.OK
    assert sc.get_state()["x"][:, 1].min() < y0


def test_fem_refusals_in_the_oracle():
    import oracle
    s = _fem_spec(linear_solver=abi.SOLVER_MINRES_ID)
    with pytest.raises(RuntimeError):
        oracle.OracleScene(s)
    s = _fem_spec()
    s.material = np.full(s.n_tets, abi.MATERIAL_ARAP, dtype=np.int32)
    with pytest.raises(RuntimeError):
        oracle.OracleScene(s)
