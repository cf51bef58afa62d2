"""GPU standard-FEM "stretch" variable (Stretch, src/variables/stretch.cpp)
against the oracle, and its refusals."""
import numpy as np
import pytest

from mfem_gb300 import abi, configs


def bbox_diag(x):
    return float(np.linalg.norm(x.max(axis=0) - x.min(axis=0)))


def _spec(prec=abi.PRECISION_FP64, material=abi.MATERIAL_SNH, **kw):
    s = configs.beam_c1(precision=prec, formulation=abi.FORMULATION_STRETCH,
                        pcg_kernel=abi.PCG_KERNEL_FUSED, **kw)
    s.material = np.full(s.n_tets, material, dtype=np.int32)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("prec,material,tol", [
    (abi.PRECISION_FP64, abi.MATERIAL_SNH, 1e-6),
    (abi.PRECISION_FP64, abi.MATERIAL_NH, 1e-6),
    (abi.PRECISION_MIXED, abi.MATERIAL_SNH, 1e-4),
])
def test_fem_steps_match_oracle(gpu_lib, prec, material, tol):
    """C1's Newton loop runs to |dx| < 1e-10, where the line search compares
    energies equal to rounding: both sides may halve until a rounding-level
    decrease appears or report a failed line search (the reference's
    MAX_ITERATIONS_REACHED), so the states agree to the iteration's noise."""
    import oracle
    from mfem_gb300 import gpu
    sp = _spec(prec, material)
    o = oracle.OracleScene(_spec(abi.PRECISION_FP64, material))
    g = gpu.Scene(sp)
    for _ in range(20):
        so, sg = o.step(), g.step()
        assert sg.status in (abi.OK, abi.ERR_LS_FAILED)
    xo, xg = o.get_state()["x"], g.get_state()["x"]
    assert np.abs(xg - xo).max() <= tol * bbox_diag(xo)
    assert np.abs(xo - sp.V_rest).max() > 1e-3 * bbox_diag(xo)   # it moved
    g.close()


@pytest.mark.gpu
def test_fem_batch_equals_alone(gpu_lib):
    from mfem_gb300 import gpu
    specs = [_spec(abi.PRECISION_MIXED), _spec(abi.PRECISION_MIXED, abi.MATERIAL_NH)]
    alone = []
    for sp in specs:
        s = gpu.Scene(sp)
        for _ in range(4):
            s.step()
        alone.append(s.get_state()["x"])
        s.close()
    scenes = [gpu.Scene(sp) for sp in specs]
    b = gpu.Batch(scenes)
    for _ in range(4):
        b.step()
    for s, ref in zip(scenes, alone):
        assert np.array_equal(s.get_state()["x"], ref)
    b.close()
    for s in scenes:
        s.close()


@pytest.mark.gpu
def test_fem_refusals(gpu_lib):
    from mfem_gb300 import gpu
    with pytest.raises(RuntimeError):
        gpu.Scene(_spec(linear_solver=abi.SOLVER_MINRES_ID))
    with pytest.raises(RuntimeError):
        gpu.Scene(_spec(material=abi.MATERIAL_COROT))
    a = gpu.Scene(_spec(abi.PRECISION_MIXED))
    b = gpu.Scene(configs.beam_c1(precision=abi.PRECISION_MIXED, pcg_kernel=abi.PCG_KERNEL_FUSED))
    with pytest.raises(RuntimeError):
        gpu.Batch([a, b])
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [abi.BC_STRETCH, abi.BC_TWIST])
def test_fem_boundary_scripts_match_oracle(gpu_lib, bc):
    import oracle
    from mfem_gb300 import gpu
    from mfem_gb300.desc import SceneSpec
    from mfem_gb300.meshgen import cube_grid, enu_to_lame
    V, T = cube_grid(6, 2, 2, 0.1)
    lam, mu = enu_to_lame(1e5, 0.4)
    sp = SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                   bc_type=bc, bc_axis=0, bc_ratio=0.05, bc_velocity=0.2, dt=1 / 60,
                   max_newton_iterations=30, iterative_solver_tolerance=1e-10,
                   max_iterative_solver_iters=2000, newton_residual_tolerance=1e-9,
                   precision=abi.PRECISION_FP64, formulation=abi.FORMULATION_STRETCH)
    o, g = oracle.OracleScene(sp), gpu.Scene(sp)
    for _ in range(4):
        o.step()
        g.step()
    xo = o.get_state()["x"]
    assert np.abs(g.get_state()["x"] - xo).max() <= 1e-6 * bbox_diag(xo)
    g.close()
