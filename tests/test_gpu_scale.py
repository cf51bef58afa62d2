"""Parity at the benchmark workloads' own sizes: the mixed path (FP32
element work, float-float reductions) against the all-FP64 GPU path and,
where the oracle finishes in seconds, against the FP64 oracle.

Bounds (those the workloads state): converged positions within 1e-6 of the
bounding-box diagonal; per-element quantities at the same state within
1e-5 relative (norm-wise over the scene).  Measured on a GB300: C3 mixed
vs FP64 1e-7 of the diagonal over six steps, C2 2e-9, the C4 mix 1.5e-9;
per-element S, dS/dF, g, H, Aloc within 2e-7.

* C3 (30^3 cubes, 135k tets, nu = 0.495, per-element E log-uniform over
  three decades, the x-max face compressed 50% over 20 steps): five steps;
  the first two also against the oracle.  Its first step is a stress case
  for both paths (the face moves 7.5 mm at once): the mixed path may end it
  on the line-search limit and the FP64 path on the PCG limit, with the
  positions still within the bound.
* C2 (60^3 cubes, 1.08M tets): three steps.
* C4 (64 scenes of 4..30 cubes a side, random materials): two steps of the
  batched mix, each scene against its FP64 twin.
"""
import numpy as np
import pytest

from mfem_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu

POS_BOUND = 1e-6   # of the bounding-box diagonal
ELEM_BOUND = 1e-5  # relative, norm-wise over the scene


def diag(x):
    return float(np.linalg.norm(np.ptp(x, axis=0)))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def elem_check(mixed, fp64, dt):
    """Per-element quantities of both paths at the FP64 scene's state."""
    st = fp64.get_state()
    mixed.set_state(x=st["x"], v=st["v"], s=st["s"], R=st["R"])
    em, ef = mixed.elem_update(st["x"], dt), fp64.elem_update(st["x"], dt)
    for k in ("R", "S", "dSdF", "g", "H", "Aloc"):
        assert rel(em[k], ef[k]) < ELEM_BOUND, (k, rel(em[k], ef[k]))


def test_c3_precision_stress_mixed_vs_fp64_and_oracle(gpu_lib):
    import oracle
    kw = dict(pcg_kernel=abi.PCG_KERNEL_AUTO)
    sm, sf = configs.stress_c3(**kw), configs.stress_c3(precision=abi.PRECISION_FP64, **kw)
    m, f, o = gpu.Scene(sm), gpu.Scene(sf), oracle.OracleScene(sf)
    ok = (abi.OK, abi.ERR_LS_FAILED, abi.ERR_CG_MAXITER)
    for k in range(5):
        a, b = m.step(), f.step()
        assert a.status in (ok if k == 0 else (abi.OK,)), (k, a.status)
        assert b.status in (ok if k == 0 else (abi.OK,)), (k, b.status)
        xm, xf = m.positions(), f.positions()
        assert np.isfinite(xm).all()
        assert np.abs(xm - xf).max() <= POS_BOUND * diag(xf), k
        if k < 2:
            c = o.step()
            assert c.status in ok
            xo = o.get_state()["x"]
            assert np.abs(xf - xo).max() <= POS_BOUND * diag(xo), k
            assert np.abs(xm - xo).max() <= POS_BOUND * diag(xo), k
    # after five steps of compression the body has moved well beyond the bound
    assert np.abs(xf - sf.V_rest).max() > 1e3 * POS_BOUND * diag(xf)
    elem_check(m, f, sm.dt)
    m.close()
    f.close()


def test_c2_cube_mixed_vs_fp64(gpu_lib):
    sm = configs.cube_c2(pcg_kernel=abi.PCG_KERNEL_AUTO)
    sf = configs.cube_c2(precision=abi.PRECISION_FP64, pcg_kernel=abi.PCG_KERNEL_AUTO)
    m, f = gpu.Scene(sm), gpu.Scene(sf)
    for k in range(3):
        a, b = m.step(), f.step()
        assert a.status == abi.OK and b.status == abi.OK, (a.status, b.status)
        xm, xf = m.positions(), f.positions()
        assert np.abs(xm - xf).max() <= POS_BOUND * diag(xf), k
    elem_check(m, f, sm.dt)
    m.close()
    f.close()


def test_c4_mix_each_scene_vs_its_fp64_twin(gpu_lib):
    kw = dict(pcg_kernel=abi.PCG_KERNEL_AUTO)
    sm = configs.batch_c4(**kw)
    sf = configs.batch_c4(precision=abi.PRECISION_FP64, **kw)
    gm, gf = [gpu.Scene(s) for s in sm], [gpu.Scene(s) for s in sf]
    bm, bf = gpu.Batch(gm), gpu.Batch(gf)
    for _ in range(2):
        a, b = bm.step(raise_on_error=False), bf.step(raise_on_error=False)
        for i in range(len(gm)):
            # a scene whose PCG needs about max_iterative_solver_iters may end a
            # solve on that limit in either path; its positions still agree
            assert a[i].status in (abi.OK, abi.ERR_LS_FAILED, abi.ERR_CG_MAXITER), i
            assert b[i].status in (abi.OK, abi.ERR_CG_MAXITER), i
            xm, xf = gm[i].positions(), gf[i].positions()
            assert np.abs(xm - xf).max() <= POS_BOUND * diag(xf), i
    bm.close()
    bf.close()
    for s in gm + gf:
        s.close()
