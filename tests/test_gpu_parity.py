"""CUDA path vs the FP64 oracle, through the C ABI.

Tolerances (written per test):
* FP64 path: per-element quantities to 1e-6 relative (the two sides differ
  only by the Procrustes stopping point, |g| < 1e-6) and 1e-9 for R, S;
  assembled system to 1e-8; positions after 100 steps within 1e-6 of the
  bounding-box diagonal.
* mixed path (FP32 element work, FP64 reductions): per-element energies,
  gradients and stretch updates within 1e-5 relative (norm-wise).
"""
import numpy as np
import pytest

import oracle
from mfem_gb300 import abi, configs, gpu
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask

pytestmark = pytest.mark.gpu

PRECS = [abi.PRECISION_FP64, abi.PRECISION_MIXED]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def bbox_diag(x):
    return np.linalg.norm(x.max(0) - x.min(0))


def deformed_state(spec, amp=0.01, seed=1):
    o = oracle.OracleScene(spec)
    x0 = o.get_state()["x"]
    rng = np.random.default_rng(seed)
    free = (spec.is_fixed == 0)[:, None] if spec.is_fixed is not None else 1.0
    return x0 + amp * rng.uniform(-1, 1, x0.shape) * free


@pytest.mark.parametrize("prec", PRECS)
def test_elem_update_parity(gpu_lib, prec):
    spec = configs.beam_c1(precision=prec)
    x = deformed_state(spec)
    o = oracle.OracleScene(spec)
    g = gpu.Scene(spec)
    # s = S(x) of the deformed state so that g = h^2 psi'(s) is non-trivial
    s_def = o.elem_update(x, spec.dt)["S"]
    o.set_state(s=s_def)
    g.set_state(s=s_def)
    eo = o.elem_update(x, spec.dt)
    eg = g.elem_update(x, spec.dt)
    tight = prec == abi.PRECISION_FP64
    assert rel(eg["R"], eo["R"]) < (1e-9 if tight else 1e-6)
    assert rel(eg["S"], eo["S"]) < (1e-9 if tight else 1e-6)
    for k in ("dSdF", "g", "H", "Aloc", "gl"):
        assert rel(eg[k], eo[k]) < (1e-6 if tight else 1e-5), k
    # Hinv is ill-conditioned where the psd projection clamps eigenvalues to
    # 1e-6 h^2; its error is about cond(H) times that of H (rounding 1e-16 in
    # FP64, 1e-7 in FP32), so it is checked on elements whose condition
    # number keeps that below the bound.
    H = eo["H"].reshape(-1, 6, 6)
    well = np.linalg.cond(H) < (1e6 if tight else 1e3)
    assert well.sum() > len(H) // 2
    assert rel(eg["Hinv"][well], eo["Hinv"][well]) < (1e-6 if tight else 1e-4)


@pytest.mark.parametrize("prec", PRECS)
def test_system_and_pcg_parity(gpu_lib, prec):
    spec = configs.beam_c1(precision=prec)
    o = oracle.OracleScene(spec)
    g = gpu.Scene(spec)
    x = deformed_state(spec, 0.005, seed=4)
    o.set_state(x=x)
    g.set_state(x=x)
    rp, col, val, rhs = g.get_system()
    rpo, colo, valo, rhso = o.get_system()
    assert np.array_equal(rp, rpo) and np.array_equal(col, colo)
    tight = prec == abi.PRECISION_FP64
    # FP64: bounded by the Procrustes stopping tolerance (|g| < 1e-6)
    assert rel(val, valo) < (1e-7 if tight else 1e-5)
    assert rel(rhs, rhso) < (1e-7 if tight else 1e-5)
    xg, itg, errg = g.pcg(rhso)
    xo, ito, erro = o.pcg(rhso)
    # the CG contract on the GPU's own matrix: |A x - b| <= tol |b| (tol 1e-8)
    n = len(rp) - 1
    Ax = np.zeros(3 * n)
    for r in range(n):
        for q in range(rp[r], rp[r + 1]):
            Ax[3 * r:3 * r + 3] += val[q] @ xg[3 * col[q]:3 * col[q] + 3]
    true_rel = np.linalg.norm(Ax - rhso) / np.linalg.norm(rhso)
    if tight:
        assert abs(itg - ito) <= 1
        assert true_rel < 1.5e-8
        # the two matrices differ by the Procrustes stopping tolerance
        assert rel(xg, xo) < 1e-6
    else:
        assert errg < 1e-7 and true_rel < 1e-5
        assert rel(xg, xo) < 1e-4


def test_beam_c1_fp64_100_steps_vs_oracle(gpu_lib):
    spec = configs.beam_c1(precision=abi.PRECISION_FP64)
    o = oracle.OracleScene(spec)
    g = gpu.Scene(spec)
    for _ in range(100):
        sg = g.step()
        so = o.step()
        assert sg.status in (abi.OK, abi.ERR_LS_FAILED)
    xg, xo = g.get_state()["x"], o.get_state()["x"]
    assert np.abs(xg - xo).max() <= 1e-6 * bbox_diag(xo)


def test_beam_mixed_residual_newton_vs_oracle(gpu_lib):
    """Mixed precision with the 1e-5 relative-residual Newton test vs the FP64
    oracle run to the same criterion."""
    kw = dict(newton_residual_tolerance=1e-5, iterative_solver_tolerance=1e-6,
              max_newton_iterations=20)
    so_spec = configs.beam_c1(precision=abi.PRECISION_FP64, **kw)
    sg_spec = configs.beam_c1(precision=abi.PRECISION_MIXED, **kw)
    o = oracle.OracleScene(so_spec)
    g = gpu.Scene(sg_spec)
    for _ in range(20):
        st = g.step()
        o.step()
        assert st.residual <= 1e-5 * st.residual0 * 1.0001 or st.newton_iterations == 20
    xg, xo = g.get_state()["x"], o.get_state()["x"]
    # the workloads' bound; measured on a GB300: 1e-8 of the diagonal
    assert np.abs(xg - xo).max() <= 1e-6 * bbox_diag(xo)


def test_beam_c1_mixed_100_steps_vs_oracle(gpu_lib):
    """C1 as stated (100 steps, PCG to 1e-8) in the mixed path (FP32
    element work, float-float reductions) against the FP64 oracle: within
    1e-6 of the bounding-box diagonal (measured on a GB300: 1.8e-8)."""
    o = oracle.OracleScene(configs.beam_c1(precision=abi.PRECISION_FP64))
    g = gpu.Scene(configs.beam_c1(precision=abi.PRECISION_MIXED))
    for _ in range(100):
        sg = g.step()
        o.step()
        assert sg.status in (abi.OK, abi.ERR_LS_FAILED, abi.ERR_CG_MAXITER)
    xg, xo = g.get_state()["x"], o.get_state()["x"]
    assert np.abs(xg - xo).max() <= 1e-6 * bbox_diag(xo)


@pytest.mark.parametrize("mtype", range(6))
def test_material_parity(gpu_lib, mtype):
    spec = configs.beam_c1(precision=abi.PRECISION_FP64, material=np.full(200, mtype, np.int32))
    x = deformed_state(spec, 0.003, seed=mtype)
    o = oracle.OracleScene(spec)
    g = gpu.Scene(spec)
    s_def = o.elem_update(x, spec.dt)["S"]
    o.set_state(s=s_def)
    g.set_state(s=s_def)
    eo = o.elem_update(x, spec.dt)
    eg = g.elem_update(x, spec.dt)
    for k in ("g", "H", "Aloc", "gl"):
        assert rel(eg[k], eo[k]) < 1e-6, k
    o2, g2 = oracle.OracleScene(spec), gpu.Scene(spec)
    for _ in range(3):
        o2.step()
        g2.step()
    xo = o2.get_state()["x"]
    assert np.abs(g2.get_state()["x"] - xo).max() <= 1e-6 * bbox_diag(xo)


def _bc_spec(bc, prec=abi.PRECISION_FP64, bdf=1):
    V, T = cube_grid(6, 2, 2, 0.1)
    lam, mu = enu_to_lame(1e5, 0.4)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     bc_type=bc, bc_axis=0, bc_ratio=0.05, bc_velocity=0.2, dt=1 / 60,
                     body_force=(0.0, -9.8, 0.0), bdf_order=bdf, max_newton_iterations=30,
                     iterative_solver_tolerance=1e-10, max_iterative_solver_iters=2000,
                     newton_residual_tolerance=1e-9, precision=prec)


@pytest.mark.parametrize("bc", [abi.BC_NULL, abi.BC_HANG, abi.BC_HANGENDS, abi.BC_ONEPOINT,
                                abi.BC_STRETCH, abi.BC_TWIST, abi.BC_BEND, abi.BC_SCALEF,
                                abi.BC_PINMIN, abi.BC_COMPRESS])
def test_boundary_scripts_vs_oracle(gpu_lib, bc):
    spec = _bc_spec(bc)
    o, g = oracle.OracleScene(spec), gpu.Scene(spec)
    assert o.n_free == g.n_free
    for _ in range(4):
        o.step()
        g.step()
    xo = o.get_state()["x"]
    assert np.abs(g.get_state()["x"] - xo).max() <= 1e-6 * bbox_diag(xo)


@pytest.mark.parametrize("bdf", [2, 3])
def test_bdf_orders_vs_oracle(gpu_lib, bdf):
    spec = _bc_spec(abi.BC_PINMIN, bdf=bdf)
    o, g = oracle.OracleScene(spec), gpu.Scene(spec)
    for _ in range(5):
        o.step()
        g.step()
    so, sg = o.get_state(), g.get_state()
    assert np.abs(sg["x"] - so["x"]).max() <= 1e-6 * bbox_diag(so["x"])
    assert np.abs(sg["v"] - so["v"]).max() <= 1e-4 * (np.abs(so["v"]).max() + 1e-9)


def test_block_jacobi_solver_converges_to_same_state(gpu_lib):
    a = configs.beam_c1(precision=abi.PRECISION_FP64)
    b = configs.beam_c1(precision=abi.PRECISION_FP64, linear_solver=abi.SOLVER_GPU_PCG_BLOCK)
    ga, gb = gpu.Scene(a), gpu.Scene(b)
    ia = ib = 0
    for _ in range(5):
        ia += ga.step().cg_iterations
        ib += gb.step().cg_iterations
    xa = ga.get_state()["x"]
    assert np.abs(gb.get_state()["x"] - xa).max() <= 1e-6 * bbox_diag(xa)
    assert ib <= ia


def _three_specs(prec):
    out = []
    for k, dims in enumerate([(5, 3, 2), (3, 4, 4), (7, 2, 3)]):
        V, T = cube_grid(*dims, 0.05)
        lam, mu = enu_to_lame(2e5 * (k + 1), 0.3 + 0.05 * k)
        out.append(SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                             is_fixed=face_mask(V, k % 3, "min"), dt=1 / 60,
                             max_newton_iterations=6, iterative_solver_tolerance=1e-6,
                             newton_residual_tolerance=1e-5, precision=prec))
    return out


@pytest.mark.parametrize("prec", PRECS)
def test_batch_result_equals_alone(gpu_lib, prec):
    """Each scene's result is bitwise the same alone and in the mix."""
    alone = []
    for spec in _three_specs(prec):
        s = gpu.Scene(spec)
        for _ in range(3):
            s.step()
        alone.append(s.get_state())
    scenes = [gpu.Scene(spec) for spec in _three_specs(prec)]
    batch = gpu.Batch(scenes)
    for _ in range(3):
        stats = batch.step()
        assert all(st.status in (abi.OK, abi.ERR_LS_FAILED) for st in stats)
    for s, ref in zip(scenes, alone):
        st = s.get_state()
        for k in ("x", "v", "s", "R"):
            assert np.array_equal(st[k], ref[k]), k


def test_rerun_is_bitwise_deterministic(gpu_lib):
    spec = configs.beam_c1(precision=abi.PRECISION_MIXED, newton_residual_tolerance=1e-5,
                           iterative_solver_tolerance=1e-5)
    runs = []
    for _ in range(2):
        s = gpu.Scene(spec)
        for _ in range(5):
            s.step()
        runs.append(s.get_state())
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


@pytest.mark.parametrize("prec", PRECS)
def test_persistent_and_split_pcg_are_bitwise_equal(gpu_lib, prec):
    """The one-launch cooperative PCG and the two-launches-per-iteration PCG
    run the same arithmetic in the same order: same states, same counts.
    The batch has more PCG tiles than one, so the grid barrier is used."""
    states, counts = [], []
    for kern in (abi.PCG_KERNEL_PERSISTENT, abi.PCG_KERNEL_SPLIT):
        specs = _three_specs(prec)
        V, T = cube_grid(12, 6, 6, 0.05)  # 637 free vertices: 3 PCG tiles
        lam, mu = enu_to_lame(1e5, 0.4)
        specs.append(SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                               is_fixed=face_mask(V, 0, "min"), dt=1 / 60, max_newton_iterations=8,
                               iterative_solver_tolerance=1e-6, newton_residual_tolerance=1e-6,
                               precision=prec))
        for sp in specs:
            sp.pcg_kernel = kern
        scenes = [gpu.Scene(sp) for sp in specs]
        batch = gpu.Batch(scenes)
        cg = []
        for _ in range(3):
            cg.append([st.cg_iterations for st in batch.step()])
        states.append([s.get_state() for s in scenes])
        counts.append(cg)
    assert counts[0] == counts[1]
    assert sum(map(sum, counts[0])) > 0
    for a, b in zip(*states):
        for k in ("x", "v", "s", "R"):
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("prec", PRECS)
def test_fused_pcg_matches_two_reduction_pcg(gpu_lib, prec):
    """The single-reduction PCG (one launch per iteration) and Eigen's PCG
    iteration agree to the rounding of the path: same Newton and PCG counts
    (within one PCG iteration per solve) and the same states."""
    res = {}
    for kern in (abi.PCG_KERNEL_SPLIT, abi.PCG_KERNEL_FUSED):
        spec = configs.beam_c1(precision=prec, pcg_kernel=kern)
        if prec == abi.PRECISION_MIXED:
            spec.iterative_solver_tolerance = 1e-5
            spec.newton_residual_tolerance = 1e-5
        s = gpu.Scene(spec)
        its = []
        for _ in range(10):
            st = s.step()
            its.append((st.newton_iterations, st.cg_iterations))
        res[kern] = (s.get_state()["x"], its)
    xa, ia = res[abi.PCG_KERNEL_SPLIT]
    xb, ib = res[abi.PCG_KERNEL_FUSED]
    tol = 1e-9 if prec == abi.PRECISION_FP64 else 1e-5
    assert np.abs(xa - xb).max() <= tol * bbox_diag(xa)
    print("two-reduction", ia, "single-reduction", ib)
    na, nb = sum(n for n, _ in ia), sum(n for n, _ in ib)
    ca, cb = sum(c for _, c in ia), sum(c for _, c in ib)
    if prec == abi.PRECISION_FP64:
        # a stopping test that sits at its threshold may flip by one iteration
        assert all(abs(p - q) <= 1 for (p, _), (q, _) in zip(ia, ib))
        assert abs(ca - cb) <= 0.05 * ca + 10
    else:
        # FP32 Newton decisions at a 1e-5 residual are rounding-sensitive, and
        # the two-reduction form replaces its recursive residual by the true
        # one every few iterations (the single-reduction form does not), so
        # their PCG counts differ on an ill-conditioned beam
        assert abs(na - nb) <= 0.25 * na + 2


@pytest.mark.gpu
def test_auto_pcg_form_by_tile_count(gpu_lib):
    """AUTO runs the fused form for a one-tile beam and the split form for a
    mid-size cube, bitwise like choosing that form directly."""
    from mfem_gb300 import gpu

    def run(spec):
        s = gpu.Scene(spec)
        b = s.solo_batch_handle()
        gpu.set_profiling(b, True)
        for _ in range(2):
            s.step()
        ks = gpu.kernel_stats(b)
        x = s.get_state()["x"]
        s.close()
        return x, ks["k_cgf_iter"][1], ks["k_cg_spmv"][1]

    beam = lambda k: configs.beam_c1(precision=abi.PRECISION_MIXED, pcg_kernel=k)
    xa, fa, sa = run(beam(abi.PCG_KERNEL_AUTO))
    xf, _, _ = run(beam(abi.PCG_KERNEL_FUSED))
    assert fa > 0 and sa == 0 and np.array_equal(xa, xf)
    cube = lambda k: configs.cube_c2(n=20, pcg_kernel=k)   # 40,000 tets: 36 PCG tiles
    xa, fa, sa = run(cube(abi.PCG_KERNEL_AUTO))
    xs, _, _ = run(cube(abi.PCG_KERNEL_SPLIT))
    assert fa == 0 and sa > 0 and np.array_equal(xa, xs)


@pytest.mark.parametrize("prec", PRECS)
def test_fused_pcg_with_block_jacobi(gpu_lib, prec):
    """The fused form keeps r, w, s unscaled under the 3x3 block-Jacobi
    preconditioner (the scaled form is for Jacobi); both reach the split
    form's states."""
    res = {}
    for kern in (abi.PCG_KERNEL_SPLIT, abi.PCG_KERNEL_FUSED):
        spec = configs.beam_c1(precision=prec, pcg_kernel=kern, linear_solver=abi.SOLVER_GPU_PCG_BLOCK)
        s = gpu.Scene(spec)
        for _ in range(5):
            assert s.step().status in (abi.OK, abi.ERR_LS_FAILED)
        res[kern] = s.get_state()["x"]
        s.close()
    xa, xb = res[abi.PCG_KERNEL_SPLIT], res[abi.PCG_KERNEL_FUSED]
    tol = 1e-7 if prec == abi.PRECISION_FP64 else 1e-5
    assert np.abs(xa - xb).max() <= tol * bbox_diag(xa)
