"""The 2-D path's descriptor options on the GPU against the 2-D oracle:
per-triangle density, initial velocities, a caller's pin mask, BDF3, the
Newton residual test, and a scene with every vertex pinned."""
import numpy as np
import pytest

from mfem_gb300 import abi
from tests.test_gpu_tri2d import _bbox, _run_pair, spec2


@pytest.mark.gpu
def test_density_velocity_and_pin_mask(gpu_lib):
    rng = np.random.default_rng(31)
    sp = spec2(10, 3, bc_type=abi.BC_NULL)
    nv, nt = sp.n_vertices, sp.n_tris
    sp.density = 500.0 + 1000.0 * rng.uniform(size=nt)
    sp.v_init = 0.2 * rng.uniform(-1, 1, (nv, 2))
    fixed = np.zeros(nv, np.int32)
    fixed[[0, 10]] = 1                      # the two bottom corners
    sp.is_fixed = fixed
    so, sg, g = _run_pair(sp, 4)
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * _bbox(so["x"])
    assert np.abs(sg["v"] - so["v"]).max() < 1e-6 * np.abs(so["v"]).max()
    g.close()


@pytest.mark.gpu
def test_bdf3_matches_oracle(gpu_lib):
    so, sg, g = _run_pair(spec2(10, 3, bdf_order=3), 5)
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * _bbox(so["x"])
    g.close()


@pytest.mark.gpu
def test_newton_residual_test_matches_oracle(gpu_lib):
    """With newton_residual_tolerance the loop stops on |rhs_k| <= tol |rhs_0|;
    both sides take the same Newton counts."""
    sp = spec2(10, 3, max_newton_iterations=20, newton_residual_tolerance=1e-4)
    so, sg, g = _run_pair(sp, 4)
    assert np.abs(sg["x"] - so["x"]).max() < 1e-7 * _bbox(so["x"])
    g.close()


@pytest.mark.gpu
def test_all_pinned_scene_follows_its_script(gpu_lib):
    """No free vertex: no PCG runs and the positions are the script's (the
    line search over s alone may end either way at rounding level, so only
    the positions are compared)."""
    import oracle
    from mfem_gb300.tri2d import Tri2dScene
    sp = spec2(4, 2, bc_type=abi.BC_STRETCH, bc_ratio=0.1, bc_velocity=0.2)
    sp.is_fixed = np.ones(sp.n_vertices, np.int32)
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    assert g.n_free == 0
    for _ in range(2):
        so, sg = o.step(), g.step()
        assert sg.status in (abi.OK, abi.ERR_LS_FAILED) and sg.cg_iterations == 0
    assert np.array_equal(g.get_state()["x"], o.get_state()["x"])
    g.close()


@pytest.mark.gpu
def test_pcg_tolerance_above_one_runs_no_iteration(gpu_lib):
    """Eigen's test before the first iteration: with tol > 1 the threshold
    tol^2 |b|^2 exceeds |b|^2, so the solve returns dx = 0 after 0
    iterations, on both sides."""
    import oracle
    from mfem_gb300.tri2d import Tri2dScene
    sp = spec2(6, 2, iterative_solver_tolerance=2.0, max_newton_iterations=2)
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    so, sg = o.step(), g.step()
    assert so.cg_iterations == 0 and sg.cg_iterations == 0
    assert sg.status == so.status and sg.newton_iterations == so.newton_iterations
    assert np.array_equal(g.get_state()["x"], o.get_state()["x"])
    g.close()
