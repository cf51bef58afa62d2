"""The single-reduction (fused) PCG: its verified stop in the mixed path and
its kernel shapes.

* Verified stop: in FP32 the recursive residual drifts from the true one
  (on the 1M-tet cube the recursion reported 9.6e-5 while |b - A dx|/|b|
  was 6.9e-4 at tol 1e-4).  The mixed path now checks b - A dx, computed
  with exact products in float-float, before it stops, so the true residual
  of the returned dx meets the tolerance (written below: 1.01 x tol, the
  host's FP64 product against the device's float-float one).
* Shapes: the matrix streamed through registers, or staged through 2, 3 or
  4 shared-memory buffers per warp by bulk copies, with or without the L2
  keep policy, one or two slots' gathers in flight, with or without
  programmatic dependent launch.  They change only how the data moves: the
  steps are bitwise the same in every shape.
"""
import numpy as np
import pytest

from mfem_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def bsr_mul(rp, col, val, x):
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    y = np.zeros((n, 3))
    np.add.at(y, rows, np.einsum("kij,kj->ki", val, x.reshape(-1, 3)[col]))
    return y.ravel()


def cube(n, precision=abi.PRECISION_MIXED, **kw):
    return configs.cube_c2(n=n, precision=precision, pcg_kernel=abi.PCG_KERNEL_FUSED, **kw)


@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_fused_mixed_true_residual_meets_tolerance(gpu_lib, tol):
    sc = gpu.Scene(cube(20, iterative_solver_tolerance=tol, max_iterative_solver_iters=5000))
    st = sc.step()
    assert st.status == abi.OK
    rp, col, val, rhs = sc.get_system()
    dx, it, err = sc.pcg(rhs)
    assert 0 < it < 5000
    true = np.linalg.norm(rhs - bsr_mul(rp, col, val, dx)) / np.linalg.norm(rhs)
    assert err < tol                     # the reported residual is the verified one
    assert true <= 1.01 * tol, (true, err, it)
    sc.close()


@pytest.mark.parametrize("prec", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_fused_shapes_compute_the_same_bits(gpu_lib, prec):
    sc = gpu.Scene(cube(20, precision=prec))
    bh = sc.solo_batch_handle()
    sc.step()
    s0 = sc.get_state()
    shapes = [(0, 0, 1, 0), (2, 0, 1, 0), (3, 0, 1, 0), (4, 0, 1, 0), (2, 1, 1, 0), (4, 1, 1, 0),
              (4, 0, 2, 0), (4, 1, 2, 0), (2, 0, 1, 1), (4, 0, 2, 1), (3, 1, 1, 1), (8, 0, 4, 0), (8, 0, 4, 1)]
    fp64 = prec == abi.PRECISION_FP64
    ref = None
    for shape in shapes:
        gpu.set_pcg_shape(bh, *shape)
        got = gpu.get_pcg_shape(bh)
        assert got == ((min(shape[0], 2), shape[1], 1, shape[3]) if fp64 else shape)
        sc.set_state(x=s0["x"], v=s0["v"], s=s0["s"], R=s0["R"])
        stats = [sc.step() for _ in range(2)]
        assert all(s.status == abi.OK for s in stats)
        out = (sc.positions(), [(s.newton_iterations, s.cg_iterations) for s in stats])
        if ref is None:
            ref = out
        else:
            assert np.array_equal(out[0], ref[0]), shape
            assert out[1] == ref[1], shape
    sc.close()


def test_fused_shape_is_validated(gpu_lib):
    sc = gpu.Scene(cube(6))
    bh = sc.solo_batch_handle()
    from mfem_gb300._lib import MfemError
    for bad in ((1, 0, 1, 0), (5, 0, 1, 0), (-1, 0, 1, 0), (2, 2, 1, 0), (2, 0, 2, 0), (4, 0, 3, 0),
                (4, 0, 0, 0), (0, 0, 1, 1), (2, 0, 1, 2), (8, 0, 1, 0), (8, 0, 2, 0), (4, 0, 4, 0), (6, 0, 1, 0)):
        with pytest.raises(MfemError):
            gpu.set_pcg_shape(bh, *bad)
    sc.close()


@pytest.mark.parametrize("b2", [1e-20, 1e-32, 1e-38, 1e-42])
def test_fused_mixed_tiny_rhs_stays_in_range(gpu_lib, b2):
    """Right-hand sides whose per-entry squares fall below FP32's normal
    range (the float-float inner products' exponent range): the mixed path
    solves for 2^k b with 2^k from max |b_i|, so the verified stop still
    meets the tolerance, with the unscaled solve's iteration count."""
    tol = 1e-6
    sc = gpu.Scene(cube(16, iterative_solver_tolerance=tol, max_iterative_solver_iters=5000))
    sc.step()
    rp, col, val, rhs = sc.get_system()
    _, it0, _ = sc.pcg(rhs)
    b = rhs * (np.sqrt(b2) / np.linalg.norm(rhs))
    dx, it, err = sc.pcg(b)
    assert np.isfinite(dx).all() and err < tol, (it, err)
    true = np.linalg.norm(b - bsr_mul(rp, col, val, dx)) / np.linalg.norm(b)
    assert true <= 1.01 * tol, true
    assert abs(it - it0) <= max(3, it0 // 20), (it, it0)
    sc.close()


@pytest.mark.parametrize("p", [-40, 40])
def test_fused_mixed_power_of_two_scaling_is_exact(gpu_lib, p):
    """Scaling b by a power of two scales the solution by it, bitwise (2^p
    keeps every entry of b, and of the solution's float pairs, a normal
    FP32 number, so the scaling itself is exact)."""
    sc = gpu.Scene(cube(16, iterative_solver_tolerance=1e-6, max_iterative_solver_iters=5000))
    sc.step()
    rp, col, val, rhs = sc.get_system()
    dx0, it0, _ = sc.pcg(rhs)
    dx1, it1, _ = sc.pcg(rhs * 2.0 ** p)
    assert it1 == it0 and np.array_equal(dx1, dx0 * 2.0 ** p)
    sc.close()


@pytest.mark.parametrize("kern", [abi.PCG_KERNEL_FUSED, abi.PCG_KERNEL_SPLIT])
@pytest.mark.parametrize("prec", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_device_driven_pcg_loop_equals_host_checked(gpu_lib, monkeypatch, kern, prec):
    """The PCG loop as one graph (a WHILE node whose condition the device
    sets after each chunk of iterations) takes the same steps, bitwise, as
    the chunks the host checks one behind, and launches at most one chunk
    beyond the iterations of each solve."""
    sp = configs.cube_c2(n=14, precision=prec, pcg_kernel=kern)
    monkeypatch.setenv("MFEM_GB300_CG_LOOP", "0")
    host = gpu.Scene(sp)
    monkeypatch.delenv("MFEM_GB300_CG_LOOP")
    dev = gpu.Scene(sp)
    name = "k_cgf_iter" if kern == abi.PCG_KERNEL_FUSED else "k_cg_spmv"
    chunk = 8 if kern == abi.PCG_KERNEL_FUSED else 25
    l0 = gpu.kernel_stats(dev.solo_batch_handle())[name][1]
    cg = solves = 0
    for _ in range(3):
        a, b = host.step(), dev.step()
        assert (a.status, a.newton_iterations, a.cg_iterations) == (b.status, b.newton_iterations, b.cg_iterations)
        cg += b.cg_iterations
        solves += b.newton_iterations
    assert np.array_equal(host.positions(), dev.positions())
    launched = gpu.kernel_stats(dev.solo_batch_handle())[name][1] - l0
    # per solve: the iteration that meets the tolerance (not counted, as in
    # Eigen), the rest of its chunk, and in the mixed fused form up to 9
    # launches of its verified stop; a Newton pass whose residual test is
    # met at assembly enters no chunk
    extra = 9 if (kern == abi.PCG_KERNEL_FUSED and prec == abi.PRECISION_MIXED) else 0
    assert cg <= launched <= cg + solves * (chunk + 1 + extra), (launched, cg, solves)
    loop = gpu.kernel_stats(dev.solo_batch_handle())["k_cg_loop"][1]
    assert loop > 0 and gpu.kernel_stats(host.solo_batch_handle())["k_cg_loop"][1] == 0
    host.close()
    dev.close()
