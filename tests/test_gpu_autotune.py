"""The autotuner: at batch creation it times register-budget variants of
the element kernels and the fused PCG shapes on the batch's own system,
keeps the fastest, and caches the choice by size class.  Every candidate it
may pick computes the default's bits (checked here one variant at a time,
in both precisions), so a tuned scene steps exactly as an untuned one."""
import numpy as np
import pytest

from mfem_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def test_tuning_report_cache_and_identical_steps(gpu_lib, monkeypatch, tmp_path):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("MFEM_GB300_TUNE_CACHE", str(cache))
    spec = configs.cube_c2(n=16, pcg_kernel=abi.PCG_KERNEL_FUSED)
    monkeypatch.setenv("MFEM_GB300_TUNE", "force")
    tuned = gpu.Scene(spec)
    rep = gpu.tune_report(tuned.solo_batch_handle())
    assert rep["source"] == "tuned"
    for k in ("k_elem_update", "k_cgf_iter", "k_local_solve", "k_ls_energy"):
        kr = rep["kernels"][k]
        assert kr["chosen"] in kr["candidates"] and kr["tuned_ms"] <= kr["default_ms"]
        assert all(t > 0 for t in kr["candidates"].values())
    assert cache.exists() and rep["key"] in cache.read_text()
    monkeypatch.setenv("MFEM_GB300_TUNE", "0")
    plain = gpu.Scene(spec)
    assert gpu.tune_report(plain.solo_batch_handle())["source"] == "default"
    monkeypatch.setenv("MFEM_GB300_TUNE", "1")
    cached = gpu.Scene(spec)
    assert gpu.tune_report(cached.solo_batch_handle())["source"] == "cache"
    for _ in range(3):
        a, b, c = tuned.step(), plain.step(), cached.step()
        assert a.status == b.status == c.status == abi.OK
        assert a.cg_iterations == b.cg_iterations == c.cg_iterations
    assert np.array_equal(tuned.positions(), plain.positions())
    assert np.array_equal(cached.positions(), plain.positions())
    for s in (tuned, plain, cached):
        s.close()


@pytest.mark.parametrize("prec", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
@pytest.mark.parametrize("variants", [(1, 0, 0), (0, 1, 0), (0, 2, 0), (0, 0, 1)])
def test_each_register_variant_computes_the_same_bits(gpu_lib, monkeypatch, prec, variants):
    monkeypatch.setenv("MFEM_GB300_TUNE", "0")
    fp64 = prec == abi.PRECISION_FP64
    if fp64 and variants[0]:
        pytest.skip("K1 has one variant in FP64")
    spec = configs.cube_c2(n=12, precision=prec, pcg_kernel=abi.PCG_KERNEL_FUSED)
    ref, var = gpu.Scene(spec), gpu.Scene(spec)
    gpu.set_variants(var.solo_batch_handle(), *variants)
    for _ in range(3):
        a, b = ref.step(), var.step()
        assert (a.status, a.newton_iterations, a.cg_iterations) == (b.status, b.newton_iterations, b.cg_iterations)
    assert np.array_equal(ref.get_state()["s"], var.get_state()["s"])
    assert np.array_equal(ref.positions(), var.positions())
    ref.close()
    var.close()


def test_variants_are_validated(gpu_lib, monkeypatch):
    monkeypatch.setenv("MFEM_GB300_TUNE", "0")
    sc = gpu.Scene(configs.cube_c2(n=4))
    from mfem_gb300._lib import MfemError
    for bad in ((2, 0, 0), (0, 3, 0), (0, 0, 2), (-1, 0, 0)):
        with pytest.raises(MfemError):
            gpu.set_variants(sc.solo_batch_handle(), *bad)
    sc.close()
