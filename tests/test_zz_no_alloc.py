"""The allocation-free block-Jacobi PCG (mfem_gpu_bsr_pcg_noalloc) against
the scene PCG (mfem_gpu_scene_pcg) on the same assembled system.

The system is the Schur-complement matrix PMP + A_mixed and its RHS that a
scene assembles (mfem_gpu_scene_get_system), copied to device buffers that
the test owns; the entry point itself allocates nothing.  This file runs
last so that the check also covers a process in which other tests have
already used the library.
"""
import ctypes as C

import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300._lib import load

MAX_ROWS = 32768  # MFEM_NOALLOC_PCG_MAX_ROWS in include/mfem_gb300.h
TOL = 1e-10


def _noalloc(n, nnzb, rp, col, val, b, x, max_iters, tol, stream=None):
    it = C.c_int32(-1)
    err = C.c_double(-1.0)
    rc = load().mfem_gpu_bsr_pcg_noalloc(n, nnzb, rp, col, val, b, x, max_iters, tol, stream,
                                         C.byref(it), C.byref(err))
    return rc, it.value, err.value


def test_noalloc_rejects_oversize_and_bad_arguments():
    # Rejected on the host before any device call: runs without a GPU.
    rc, it, _ = _noalloc(MAX_ROWS + 1, 0, None, None, None, None, None, 10, 1e-8)
    assert rc == abi.ERR_CAPACITY and it == 0
    assert _noalloc(-1, 0, None, None, None, None, None, 10, 1e-8)[0] == abi.ERR_INVALID
    assert _noalloc(8, 0, None, None, None, None, None, 10, float("nan"))[0] == abi.ERR_INVALID
    assert _noalloc(0, 0, None, None, None, None, None, 10, 1e-8)[0] == abi.OK


def _system_spec():
    from mfem_gb300.desc import SceneSpec
    from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask
    V, T = cube_grid(20, 6, 6, 0.05)  # 1029 vertices, 980 free: 4 tiles of 256 rows
    lam, mu = enu_to_lame(1e6, 0.45)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, 0, "min"), density_const=1000.0, dt=1.0 / 60.0,
                     body_force=(0.0, -9.8, 0.0), max_newton_iterations=10,
                     iterative_solver_tolerance=TOL, max_iterative_solver_iters=3000,
                     linear_solver=abi.SOLVER_GPU_PCG_BLOCK, precision=abi.PRECISION_FP64)


def _bsr_matvec(rp, col, val, x):
    n = len(rp) - 1
    xb = x.reshape(-1, 3)
    y = np.zeros((n, 3))
    rows = np.repeat(np.arange(n), np.diff(rp))
    np.add.at(y, rows, np.einsum("kij,kj->ki", val, xb[col]))
    return y.ravel()


@pytest.mark.gpu
def test_noalloc_pcg_matches_scene_pcg():
    import torch
    from mfem_gb300 import gpu

    scene = gpu.Scene(_system_spec())
    scene.step()  # a deformed state, so that the rotations are not the identity
    rp, col, val, rhs = scene.get_system()
    n, nnzb = scene.n_free, scene.nnzb
    assert n > 256 and n <= MAX_ROWS
    x_ref, it_ref, err_ref = scene.pcg(rhs)
    assert err_ref <= TOL

    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(rp).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(np.ascontiguousarray(val).ravel()).to(dev)
    d_b = torch.from_numpy(rhs).to(dev)
    d_x = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    bnorm = np.linalg.norm(rhs)
    xs = []
    for call in range(2):  # two calls in a row on the same scratch
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc, it, err = _noalloc(n, nnzb, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                               d_b.data_ptr(), d_x.data_ptr(), 3000, TOL)
        assert rc == abi.OK, rc
        if call > 0:
            # Nothing was allocated on the device by the call.  (On the first
            # call the CUDA runtime may still be loading the library's device
            # code and its static scratch, which is the library's fixed
            # footprint, not an allocation of the call.)
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        x = d_x.cpu().numpy()
        assert np.isfinite(x).all()
        assert err <= TOL
        assert abs(it - it_ref) <= max(2, it_ref // 50)
        # Same system, same iteration, different rounding of the reductions.
        assert np.abs(x - x_ref).max() <= 1e-7 * np.abs(x_ref).max()
        true_res = np.linalg.norm(rhs - _bsr_matvec(rp, col, val, x)) / bnorm
        assert true_res <= 10 * TOL
        xs.append(x)
    assert np.array_equal(xs[0], xs[1])  # deterministic reductions


@pytest.mark.gpu
def test_noalloc_pcg_maxiter_and_singular_block():
    import torch
    from mfem_gb300 import gpu

    scene = gpu.Scene(_system_spec())
    rp, col, val, rhs = scene.get_system()
    n, nnzb = scene.n_free, scene.nnzb
    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(rp).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(np.ascontiguousarray(val).ravel()).to(dev)
    d_b = torch.from_numpy(rhs).to(dev)
    d_x = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc, it, err = _noalloc(n, nnzb, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                           d_b.data_ptr(), d_x.data_ptr(), 3, TOL)
    assert rc == abi.ERR_CG_MAXITER and it == 3 and err > TOL
    # No iteration allowed and b above the threshold: stopped on max_iters,
    # with x = 0 (Eigen reports NoConvergence here)
    rc, it, err = _noalloc(n, nnzb, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                           d_b.data_ptr(), d_x.data_ptr(), 0, TOL)
    assert rc == abi.ERR_CG_MAXITER and it == 0 and err == 1.0
    assert not d_x.any().item()
    # A host pointer is rejected before any launch.
    host_b = np.ascontiguousarray(rhs)
    rc, _, _ = _noalloc(n, nnzb, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                        host_b.ctypes.data, d_x.data_ptr(), 50, TOL)
    assert rc == abi.ERR_INVALID
    # A zero diagonal block is reported, not divided by.
    bad = np.ascontiguousarray(val).copy()
    diag = [k for k in range(rp[0], rp[1]) if col[k] == 0][0]
    bad[diag] = 0.0
    d_bad = torch.from_numpy(bad.ravel()).to(dev)
    torch.cuda.synchronize()
    rc, it, _ = _noalloc(n, nnzb, d_rp.data_ptr(), d_col.data_ptr(), d_bad.data_ptr(),
                         d_b.data_ptr(), d_x.data_ptr(), 50, TOL)
    assert rc == abi.ERR_INVALID and it == 0
