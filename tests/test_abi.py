"""The C ABI library: builds, loads without a GPU, exports every symbol the
header declares, and its structs have the layout the ctypes mirror assumes."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

from mfem_gb300 import _lib, abi

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_library_exports_every_header_symbol(gpu_lib):
    names = _lib.header_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(gpu_lib, n), n
    assert set(names) == set(_lib.SIGNATURES)


def test_abi_version_and_status_strings(gpu_lib):
    assert gpu_lib.mfem_gpu_abi_version() == abi.ABI_VERSION
    for code in range(12):
        assert gpu_lib.mfem_gpu_status_string(code)


def _c_layout(struct, fields):
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "mfem_gb300.h"', 'int main(void){']
    src.append(f'printf("%zu\\n", sizeof({struct}));')
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof({struct}, {f}));')
    src.append('return 0;}')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write("\n".join(src))
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    return [int(v) for v in out]


@pytest.mark.parametrize("cname,py", [("mfem_scene_desc", abi.SceneDesc),
                                      ("mfem_step_stats", abi.StepStats)])
def test_struct_layout_matches_header(cname, py):
    fields = [n for n, _ in py._fields_]
    cfields = ["lambda" if f == "lam" else f for f in fields]
    got = _c_layout(cname, cfields)
    assert got[0] == C.sizeof(py)
    for f, off in zip(fields, got[1:]):
        assert getattr(py, f).offset == off, f


def test_no_device_fails_loudly_without_gpu(gpu_lib):
    """On a machine without a GPU, scene creation reports MFEM_ERR_NO_DEVICE
    instead of falling back to a CPU path."""
    import numpy as np
    from mfem_gb300 import configs
    from mfem_gb300.desc import make_desc
    n = C.c_int32(0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = None
    if has_gpu:
        pytest.skip("a GPU is present")
    d = make_desc(configs.beam_c1())
    h = C.c_void_p()
    rc = gpu_lib.mfem_gpu_scene_create(C.addressof(d.struct), C.byref(h))
    assert rc == abi.ERR_NO_DEVICE


@pytest.mark.gpu
def test_bounded_wait_runs_out_and_the_context_stays_usable(gpu_lib):
    """A grid barrier that misses an arrival (a lost peer block) ends after
    its limit with MFEM_ERR_TIMEOUT instead of hanging; scenes still run."""
    from mfem_gb300 import configs, gpu
    ms = C.c_double(0.0)
    rc = gpu_lib.mfem_gpu_selftest_bounded_wait(C.byref(ms))
    assert rc == abi.ERR_TIMEOUT
    assert 500.0 < ms.value < 10000.0
    s = gpu.Scene(configs.beam_c1())
    assert s.step().status in (abi.OK, abi.ERR_LS_FAILED)
    s.close()


def test_c_caller_links_against_the_library(gpu_lib, tmp_path):
    """A plain C99 program (the kind of caller the reference's build would
    add) includes the header, links libmfem_gb300.so and calls through it:
    the 2-D create reports MFEM_ERR_NO_DEVICE without a GPU, MFEM_OK with one."""
    import shutil
    src = tmp_path / "caller.c"
    src.write_text(r'''
#include <stdio.h>
#include "mfem_gb300.h"
int main(void) {
  double V[6] = {0, 0, 1, 0, 0, 1};
  int32_t T[3] = {0, 1, 2};
  double mu = 1, la = 1;
  mfem_tri2d_desc d = {0};
  d.n_vertices = 3; d.n_tris = 1; d.V_rest = V; d.tris = T; d.mu = &mu; d.lambda = &la;
  d.density_const = 1000; d.dt = 0.01; d.bdf_order = 1; d.max_newton_iterations = 1;
  d.max_linesearch_iterations = 1; d.max_iterative_solver_iters = 10;
  d.iterative_solver_tolerance = 1e-8; d.linear_solver = MFEM_SOLVER_EIGEN_CG_DIAG;
  mfem_tri2d* s = 0;
  int rc = mfem_gpu_tri2d_create(&d, &s);
  if (rc == MFEM_OK) mfem_gpu_tri2d_destroy(s);
  printf("%d %d\n", mfem_gpu_abi_version(), rc);
  return 0;
}
''')
    libdir = os.path.join(ROOT, "mfem_gb300", "_build")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")
    exe = str(tmp_path / "caller")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lmfem_gb300", f"-Wl,-rpath,{libdir}",
                    f"-Wl,-rpath-link,{cudalib}", "-o", exe], check=True)
    ver, rc = (int(v) for v in subprocess.run([exe], capture_output=True, text=True,
                                              check=True).stdout.split())
    assert ver == abi.ABI_VERSION
    assert rc in (abi.OK, abi.ERR_NO_DEVICE)
    try:
        import torch
        if not torch.cuda.is_available():
            assert rc == abi.ERR_NO_DEVICE
    except ImportError:
        pass
