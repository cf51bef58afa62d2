"""Descriptor validation (mfem_gpu_scene_footprint runs it without a GPU):
inputs the device path must never see are refused on the host with the
ABI's status codes (the reference exits or prints "unimplemented" there)."""
import ctypes as C

import numpy as np
import pytest

from mfem_gb300 import abi, configs
from mfem_gb300.desc import make_desc


def _footprint_status(lib, spec, **desc_overrides):
    d = make_desc(spec)
    for k, v in desc_overrides.items():
        setattr(d.struct, k, v)
    b = C.c_int64(0)
    return lib.mfem_gpu_scene_footprint(C.addressof(d.struct), C.byref(b)), b.value


def test_valid_scene_has_a_footprint(gpu_lib):
    rc, b = _footprint_status(gpu_lib, configs.beam_c1())
    assert rc == abi.OK and b > 0
    rc2, b2 = _footprint_status(gpu_lib, configs.beam_c1(linear_solver=abi.SOLVER_MINRES_ID))
    assert rc2 == abi.OK and b2 > b    # MINRES vectors and element data


@pytest.mark.parametrize("field,value,status", [
    ("precision", 7, abi.ERR_INVALID),
    ("formulation", 2, abi.ERR_INVALID),
    ("pcg_kernel", 9, abi.ERR_INVALID),
    ("bdf_order", 0, abi.ERR_INVALID),
    ("bdf_order", 7, abi.ERR_INVALID),
    ("dt", 0.0, abi.ERR_INVALID),
    ("bc_axis", 3, abi.ERR_INVALID),
    ("max_newton_iterations", -1, abi.ERR_INVALID),
    ("max_iterative_solver_iters", -1, abi.ERR_INVALID),
    ("linear_solver", abi.SOLVER_CHOLMOD, abi.ERR_UNSUPPORTED),
    ("linear_solver", abi.SOLVER_MINRES_ADMM, abi.ERR_UNSUPPORTED),
])
def test_bad_descriptor_fields(gpu_lib, field, value, status):
    rc, _ = _footprint_status(gpu_lib, configs.beam_c1(), **{field: value})
    assert rc == status


def test_bad_meshes(gpu_lib):
    s = configs.beam_c1()
    bad = s.tets.copy()
    bad[3, 2] = s.n_vertices                      # index past the last vertex
    s.tets = bad
    assert _footprint_status(gpu_lib, s)[0] == abi.ERR_INVALID
    s = configs.beam_c1()
    bad = s.tets.copy()
    bad[0, 0] = -1
    s.tets = bad
    assert _footprint_status(gpu_lib, s)[0] == abi.ERR_INVALID
    s = configs.beam_c1()
    s.material = np.full(s.n_tets, 6, dtype=np.int32)   # no such material
    assert _footprint_status(gpu_lib, s)[0] == abi.ERR_INVALID


def test_standard_fem_refusals(gpu_lib):
    fem = dict(formulation=abi.FORMULATION_STRETCH)
    assert _footprint_status(gpu_lib, configs.beam_c1(**fem))[0] == abi.OK
    s = configs.beam_c1(**fem)
    s.material = np.full(s.n_tets, abi.MATERIAL_COROT, dtype=np.int32)
    assert _footprint_status(gpu_lib, s)[0] == abi.ERR_UNSUPPORTED
    s = configs.beam_c1(linear_solver=abi.SOLVER_MINRES_ID, **fem)
    assert _footprint_status(gpu_lib, s)[0] == abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("rc", [abi.ERR_NONFINITE, abi.ERR_PROCRUSTES])
def test_scene_step_returns_numerical_failures_on_request(gpu_lib, monkeypatch, rc):
    """Scene.step(raise_on_error=False) hands a numerical failure back as the
    step's status (the batched forms retire such a scene); by default it
    raises.  A CUDA error, a timed-out wait or an invalid call raises either
    way.  The library's step entry point is faked: this is host logic."""
    from mfem_gb300 import gpu
    from mfem_gb300._lib import MfemError

    class FakeLib:
        def __init__(self, code):
            self.code = code

        def mfem_gpu_scene_step(self, handle, stats_ref):
            stats_ref._obj.status = self.code
            return self.code

    sc = gpu.Scene.__new__(gpu.Scene)
    sc._h = None
    monkeypatch.setattr(gpu, "load", lambda: FakeLib(rc))
    assert sc.step(raise_on_error=False).status == rc
    with pytest.raises(MfemError):
        sc.step()
    for hard in (abi.ERR_CUDA, abi.ERR_TIMEOUT, abi.ERR_INVALID):
        monkeypatch.setattr(gpu, "load", lambda hard=hard: FakeLib(hard))
        with pytest.raises(MfemError):
            sc.step(raise_on_error=False)
