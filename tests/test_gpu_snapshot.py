"""Snapshots (resume) and device checkpoints of a scene's state between steps."""
import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask


def _spec(prec, dims=(6, 3, 3), bdf=2, bc=abi.BC_HANG):
    V, T = cube_grid(*dims, 0.05)
    lam, mu = enu_to_lame(3e5, 0.4)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, 0, "min"), dt=1 / 60, bdf_order=bdf,
                     max_newton_iterations=6, iterative_solver_tolerance=1e-6,
                     newton_residual_tolerance=1e-6, precision=prec, pcg_kernel=abi.PCG_KERNEL_FUSED)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_resume_from_snapshot_is_bitwise(gpu_lib, prec):
    from mfem_gb300 import gpu
    a = gpu.Scene(_spec(prec))
    for _ in range(3):
        a.step()
    snap = a.snapshot()
    for _ in range(2):
        a.step()
    b = gpu.Scene(_spec(prec))
    b.restore(snap)
    for _ in range(2):
        b.step()
    sa, sb = a.get_state(), b.get_state()
    for k in ("x", "v", "s", "R"):
        assert np.array_equal(sa[k], sb[k]), k
    a.close()
    b.close()


@pytest.mark.gpu
def test_rollback_retakes_the_same_step(gpu_lib):
    from mfem_gb300 import gpu
    a = gpu.Scene(_spec(abi.PRECISION_MIXED, bdf=3))
    for _ in range(2):
        a.step()
    a.checkpoint()
    a.step()
    first = a.get_state()
    a.rollback()
    a.step()
    again = a.get_state()
    for k in ("x", "v", "s", "R"):
        assert np.array_equal(first[k], again[k]), k
    a.close()


@pytest.mark.gpu
def test_snapshot_crosses_precision(gpu_lib):
    from mfem_gb300 import gpu
    m = gpu.Scene(_spec(abi.PRECISION_MIXED))
    for _ in range(3):
        m.step()
    d = gpu.Scene(_spec(abi.PRECISION_FP64))
    d.restore(m.snapshot())
    sm, sd = m.get_state(), d.get_state()
    assert np.array_equal(sm["x"], sd["x"]) and np.array_equal(sm["v"], sd["v"])
    assert np.array_equal(sm["s"], sd["s"])
    st = d.step()
    assert st.status == abi.OK and np.isfinite(d.get_state()["x"]).all()
    other = gpu.Scene(_spec(abi.PRECISION_FP64, dims=(5, 3, 3)))
    with pytest.raises(RuntimeError):
        other.restore(m.snapshot())
    for s in (m, d, other):
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [abi.BC_TWIST, abi.BC_STRETCH])
def test_resume_continues_the_boundary_script(gpu_lib, bc):
    """The scripted pins move every step; their positions travel in the
    snapshot, so a resumed scene keeps following the script bitwise."""
    from mfem_gb300 import gpu
    V, T = cube_grid(6, 2, 2, 0.1)
    lam, mu = enu_to_lame(1e5, 0.4)
    spec = SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     bc_type=bc, bc_axis=0, bc_ratio=0.05, bc_velocity=0.2, dt=1 / 60, bdf_order=2,
                     max_newton_iterations=10, iterative_solver_tolerance=1e-8,
                     precision=abi.PRECISION_MIXED, pcg_kernel=abi.PCG_KERNEL_FUSED)
    a = gpu.Scene(spec)
    for _ in range(3):
        a.step()
    snap = a.snapshot()
    for _ in range(3):
        a.step()
    b = gpu.Scene(spec)
    b.restore(snap)
    for _ in range(3):
        b.step()
    assert np.array_equal(a.get_state()["x"], b.get_state()["x"])
    assert np.abs(a.get_state()["x"] - V).max() > 1e-3       # the pins moved
    a.close()
    b.close()
