"""Several timesteps per call, each scene at its own pace
(mfem_gpu_batch_step_n): a scene whose Newton loop has ended turns over to
its next timestep in the same call instead of waiting for the batch's
slowest scene; with the single-reduction PCG a scene does not wait for the
others' PCG or line search either (the ticked form).  Its results must be bitwise those of as many calls of the
one-step form, for scenes alone and in a mix, with scripted boundary motion
and BDF2, in both precisions."""
import numpy as np
import pytest

from mfem_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


# The single-reduction PCG runs the ticked form (every kernel gated by the
# scene's phase); the persistent PCG runs rounds of whole Newton iterations.
KERNELS = [abi.PCG_KERNEL_FUSED, abi.PCG_KERNEL_PERSISTENT]


def mix_specs(precision, kern=abi.PCG_KERNEL_FUSED):
    rng = np.random.default_rng(7)
    specs = [configs.random_scene(rng, d, precision=precision, pcg_kernel=kern)
             for d in ((4, 5, 6), (9, 6, 5), (12, 4, 4), (5, 5, 14))]
    beam = configs.beam_c1(precision=precision, bc_type=abi.BC_STRETCH, bc_ratio=0.1, bc_velocity=0.05,
                           newton_residual_tolerance=1e-5, iterative_solver_tolerance=1e-4, pcg_kernel=kern)
    specs.append(beam)
    specs[1].bdf_order = 2
    return specs


def state(scs):
    return [(s.positions(), s.get_state()["s"]) for s in scs]


@pytest.mark.parametrize("kern", KERNELS)
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_step_n_equals_single_steps_bitwise(gpu_lib, precision, kern):
    steps = 5
    specs = mix_specs(precision, kern)
    a = [gpu.Scene(s) for s in specs]
    b = [gpu.Scene(s) for s in specs]
    ba, bb = gpu.Batch(a), gpu.Batch(b)
    # the one-step form, `steps` times
    per = [[0, 0, 0, 0] for _ in specs]
    for _ in range(steps):
        for i, st in enumerate(bb.step(raise_on_error=False)):
            per[i][0] += st.newton_iterations
            per[i][1] += st.cg_iterations
            per[i][2] = max(per[i][2], st.status)
            per[i][3] += st.ls_iterations
    stats, done = ba.step_n(steps, raise_on_error=False)
    for i in range(len(specs)):
        assert stats[i].newton_iterations == per[i][0], i
        assert stats[i].cg_iterations == per[i][1], i
        assert stats[i].ls_iterations == per[i][3], i
        assert (stats[i].status == 0) == (per[i][2] == 0), i
        d = done[i]
        assert (d > 0).all() and (np.diff(d) > 0).all() and d[-1] <= stats[i].device_ms + 1e-3
    for (xa, sa), (xb, sb) in zip(state(a), state(b)):
        assert np.array_equal(xa, xb) and np.array_equal(sa, sb)
    # the scenes did not all finish their steps together
    assert len({round(float(d[-1]), 3) for d in done}) > 1
    # and one more step of each form still agrees (the pins and the BDF ring
    # were left as the one-step form leaves them)
    ba.step(raise_on_error=False)
    bb.step(raise_on_error=False)
    for (xa, _), (xb, _) in zip(state(a), state(b)):
        assert np.array_equal(xa, xb)
    ba.close()
    bb.close()


@pytest.mark.parametrize("kern", KERNELS)
def test_step_n_alone_equals_in_the_mix(gpu_lib, kern):
    specs = mix_specs(abi.PRECISION_MIXED, kern)
    mix = [gpu.Scene(s) for s in specs]
    bm = gpu.Batch(mix)
    bm.step_n(4, raise_on_error=False)
    for i, sp in enumerate(specs):
        alone = gpu.Scene(sp)
        ba = gpu.Batch([alone])
        ba.step_n(4, raise_on_error=False)
        assert np.array_equal(alone.positions(), mix[i].positions()), i
        ba.close()
        alone.close()
    bm.close()


def test_step_n_validates_its_count(gpu_lib):
    sc = gpu.Scene(configs.cube_c2(n=4))
    b = gpu.Batch([sc])
    from mfem_gb300._lib import MfemError
    for bad in (0, -1, 1025):
        with pytest.raises(MfemError):
            b.step_n(bad)
    b.close()


def test_lanes_equal_one_batch(gpu_lib):
    """The scenes split into lanes (batches stepped side by side on their own
    streams, mfem_gpu_batches_step_n) take the same steps, bitwise, as in a
    single batch of the same PCG form."""
    specs = mix_specs(abi.PRECISION_MIXED)
    a = [gpu.Scene(s) for s in specs]
    b = [gpu.Scene(s) for s in specs]
    one = gpu.Batch(a)
    lanes = gpu.Lanes(b, lanes=3)
    assert len(lanes.batches) == 3 and sorted(i for p in lanes.parts for i in p) == list(range(len(specs)))
    s1, d1 = one.step_n(4, raise_on_error=False)
    s2, d2 = lanes.step_n(4, raise_on_error=False)
    for i in range(len(specs)):
        assert (s1[i].newton_iterations, s1[i].cg_iterations, s1[i].status) == \
            (s2[i].newton_iterations, s2[i].cg_iterations, s2[i].status), i
        assert ((d1[i] >= 0) == (d2[i] >= 0)).all()
    for (xa, sa), (xb, sb) in zip(state(a), state(b)):
        assert np.array_equal(xa, xb) and np.array_equal(sa, sb)
    # a batch twice, or a scene in two of the batches, is refused
    from mfem_gb300._lib import load
    import ctypes as C
    h = lanes.batches[0].handle.value
    arr = (C.c_void_p * 2)(h, h)
    assert load().mfem_gpu_batches_step_n(arr, 2, 1, None, None) == abi.ERR_INVALID
    extra = gpu.Batch([b[lanes.parts[0][0]]])
    arr = (C.c_void_p * 2)(h, extra.handle.value)
    assert load().mfem_gpu_batches_step_n(arr, 2, 1, None, None) == abi.ERR_INVALID
    extra.close()
    lanes.close()
    one.close()
