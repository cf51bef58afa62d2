"""The serving loop on the GPU: every result equals the request served alone."""
import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.desc import SceneSpec
from mfem_gb300.meshgen import cube_grid, enu_to_lame, face_mask


def _spec(dims, E, axis, prec):
    V, T = cube_grid(*dims, 0.05)
    lam, mu = enu_to_lame(E, 0.35)
    return SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, axis, "min"), dt=1 / 60, max_newton_iterations=8,
                     iterative_solver_tolerance=1e-6, newton_residual_tolerance=1e-5,
                     precision=prec, pcg_kernel=abi.PCG_KERNEL_FUSED)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_served_results_equal_alone(gpu_lib, prec):
    from mfem_gb300 import gpu, server
    reqs = [((5, 3, 2), 2e5, 0, 3), ((3, 4, 4), 4e5, 1, 5), ((7, 2, 3), 1e5, 2, 2),
            ((4, 4, 4), 3e5, 0, 4)]
    specs = [_spec(d, E, ax, prec) for d, E, ax, _ in reqs]
    alone = []
    for sp, (_, _, _, n) in zip(specs, reqs):
        s = gpu.Scene(sp)
        for _ in range(n):
            s.step()
        alone.append(s.get_state()["x"])
        s.close()
    # a budget for about two scenes at a time: the others wait and join later
    probe = server.Server(budget_bytes=1)
    need = [gpu.footprint(sp) + probe._checkpoint_bytes(sp) for sp in specs]
    budget = int(1.5 * max(need))
    srv = server.Server(budget_bytes=budget)
    for i, (sp, (_, _, _, n)) in enumerate(zip(specs, reqs)):
        srv.submit(sp, n, arrival=0.0)
    out = srv.run(realtime=False)
    assert max(n for _, n, _ in srv.ticks) >= 2        # scenes did share ticks
    for r, ref in zip(out, alone):
        assert r.status in (abi.OK, abi.ERR_CG_MAXITER)
        assert np.array_equal(r.result["x"], ref)


@pytest.mark.gpu
def test_soft_scene_escalates_to_fp64_and_stays_finite(gpu_lib):
    """A very soft body (E = 3e4 Pa, hanging from one face) at large sag: in
    mixed precision its line search fails at step 18 and, left in mixed, the
    state diverges by step 20; served, it continues in FP64 and stays finite."""
    from mfem_gb300 import configs, gpu, server
    _, spec, _ = configs.stream_c5(duration=5.0, steps=20)[84]
    spec.pcg_kernel = abi.PCG_KERNEL_FUSED
    srv = server.Server(budget_bytes=8 * gpu.footprint(spec))
    srv.submit(spec, 20)
    (r,) = srv.run(realtime=False)
    assert r.escalated_at is not None and 10 <= r.escalated_at < 20
    assert r.steps_done == 20 and r.status in (abi.OK, abi.ERR_CG_MAXITER)
    x = r.result["x"]
    assert np.isfinite(x).all() and x[:, 1].min() > -0.3


@pytest.mark.gpu
def test_served_in_lanes_with_multi_step_ticks_equals_alone(gpu_lib):
    """Two lanes (independent loops, batches and streams in two threads) and
    ticks of up to three timesteps per instance: every result is still the
    request served alone, bitwise."""
    from mfem_gb300 import gpu, server
    reqs = [((5, 3, 2), 2e5, 0, 4), ((3, 4, 4), 4e5, 1, 5), ((7, 2, 3), 1e5, 2, 3),
            ((4, 4, 4), 3e5, 0, 6), ((6, 3, 3), 2.5e5, 1, 2)]
    specs = [_spec(d, E, ax, abi.PRECISION_MIXED) for d, E, ax, _ in reqs]
    alone = []
    for sp, (_, _, _, n) in zip(specs, reqs):
        s = gpu.Scene(sp)
        for _ in range(n):
            s.step()
        alone.append(s.get_state()["x"])
        s.close()
    srv = server.Server(budget_bytes=int(1e9), lanes=2, steps_per_tick=3)
    for sp, (_, _, _, n) in zip(specs, reqs):
        srv.submit(sp, n, arrival=0.0)
    out = srv.run(realtime=False)
    for r, ref, (_, _, _, n) in zip(out, alone, reqs):
        assert r.steps_done == n and len(r.step_ms) == n
        assert np.array_equal(r.result["x"], ref)
