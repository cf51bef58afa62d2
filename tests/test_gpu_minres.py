"""GPU "minres-indefinite-block" against the oracle's MINRES and against the
reduced (PCG + local solve) path on the same Newton systems."""
import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask


def _spec(solver, tol, iters, prec, dims=(6, 3, 3), E=2e5, axis=0, newton=3):
    V, T = cube_grid(*dims, 0.05)
    lam, mu = enu_to_lame(E, 0.4)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, axis, "min"), dt=1 / 60, max_newton_iterations=newton,
                     iterative_solver_tolerance=tol, max_iterative_solver_iters=iters,
                     linear_solver=solver, precision=prec, pcg_kernel=abi.PCG_KERNEL_FUSED)


def _run(scene, steps):
    stats = [scene.step() for _ in range(steps)]
    return stats, scene.get_state()["x"]


@pytest.mark.gpu
def test_minres_fp64_matches_oracle(gpu_lib):
    import oracle
    from mfem_gb300 import gpu
    sp = _spec(abi.SOLVER_MINRES_ID, 1e-10, 5000, abi.PRECISION_FP64)
    so, xo = _run(oracle.OracleScene(sp), 2)
    g = gpu.Scene(sp)
    sg, xg = _run(g, 2)
    disp = np.abs(xo - sp.V_rest).max()
    assert np.abs(xg - xo).max() <= 1e-7 * disp
    for a, b in zip(so, sg):
        assert a.newton_iterations == b.newton_iterations and b.status == abi.OK
        # the Krylov path is rounding-sensitive over thousands of iterations
        assert abs(a.cg_iterations - b.cg_iterations) <= 0.03 * a.cg_iterations
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,bound", [(abi.PRECISION_FP64, 1e-7), (abi.PRECISION_MIXED, 1e-4)])
def test_minres_matches_reduced_path(gpu_lib, prec, bound):
    """Both solve the same Newton system; at a tight tolerance the steps agree."""
    from mfem_gb300 import gpu
    sm = _spec(abi.SOLVER_MINRES_ID, 1e-10, 5000, prec)
    sp = _spec(abi.SOLVER_EIGEN_CG_DIAG, 1e-10, 5000, abi.PRECISION_FP64)
    a, b = gpu.Scene(sm), gpu.Scene(sp)
    _, xm = _run(a, 3)
    _, xp = _run(b, 3)
    disp = np.abs(xp - sp.V_rest).max()
    assert np.abs(xm - xp).max() <= bound * disp
    a.close()
    b.close()


@pytest.mark.gpu
def test_minres_scene_tolerance_and_batch_equals_alone(gpu_lib):
    from mfem_gb300 import gpu
    specs = [_spec(abi.SOLVER_MINRES_ID, 1e-4, 500, abi.PRECISION_MIXED, dims=d, axis=ax)
             for d, ax in (((6, 3, 3), 0), ((3, 5, 3), 1))]
    alone = []
    for sp in specs:
        s = gpu.Scene(sp)
        st, x = _run(s, 3)
        assert all(t.status == abi.OK and t.cg_error < 1e-4 for t in st)
        alone.append(x)
        s.close()
    scenes = [gpu.Scene(sp) for sp in specs]
    b = gpu.Batch(scenes)
    for _ in range(3):
        b.step()
    for s, ref in zip(scenes, alone):
        assert np.array_equal(s.get_state()["x"], ref)
    b.close()
    for s in scenes:
        s.close()


@pytest.mark.gpu
def test_batch_rejects_mixed_solvers(gpu_lib):
    from mfem_gb300 import gpu
    a = gpu.Scene(_spec(abi.SOLVER_MINRES_ID, 1e-4, 500, abi.PRECISION_MIXED))
    b = gpu.Scene(_spec(abi.SOLVER_EIGEN_CG_DIAG, 1e-4, 500, abi.PRECISION_MIXED))
    with pytest.raises(RuntimeError):
        gpu.Batch([a, b])
    a.close()
    b.close()


@pytest.mark.gpu
def test_minres_neohookean_bdf2_matches_oracle(gpu_lib):
    import oracle
    from mfem_gb300 import gpu
    sp = _spec(abi.SOLVER_MINRES_ID, 1e-10, 8000, abi.PRECISION_FP64, E=5e5)
    sp.material = np.full(sp.n_tets, abi.MATERIAL_NH, dtype=np.int32)
    sp.bdf_order = 2
    o = oracle.OracleScene(sp)
    g = gpu.Scene(sp)
    for _ in range(3):
        so, sg = o.step(), g.step()
        assert sg.status == abi.OK and so.newton_iterations == sg.newton_iterations
    xo = o.get_state()["x"]
    assert np.abs(g.get_state()["x"] - xo).max() <= 1e-7 * np.abs(xo - sp.V_rest).max()
    g.close()
