"""2-D scenes (triangle meshes in the plane) on the GPU, through the
mfem_gpu_tri2d_* entry points of libmfem_gb300.so: the DIM = 2 instance of
the timestep (Tri2DMesh + MixedStretch<2> + NewtonOptimizer<2>), FP64."""
import ctypes as C

import numpy as np

from . import abi
from ._lib import check, load
from .desc import Tri2dSpec, make_tri2d_desc

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


# the 2-D kernels in the order of the MFEM_T2_K_* ids
KERNELS = ["t2_elem", "t2_rows", "t2_norm", "t2_pcg", "t2_local", "t2_energy", "t2_esum",
           "t2_apply", "t2_history"]


class Tri2dScene:
    """One resident 2-D instance (SimState<2> + NewtonOptimizer<2>)."""

    def __init__(self, spec: Tri2dSpec):
        L = load()
        self.spec = spec
        self._desc = make_tri2d_desc(spec)
        h = C.c_void_p()
        check(L.mfem_gpu_tri2d_create(C.addressof(self._desc.struct), C.byref(h)), "tri2d_create")
        self._h = h
        nv, nt, nf, nb = (C.c_int32() for _ in range(4))
        L.mfem_gpu_tri2d_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(nf), C.byref(nb))
        self.n_vertices, self.n_tris, self.n_free, self.nnzb = nv.value, nt.value, nf.value, nb.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().mfem_gpu_tri2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, raise_on_error=False):
        st = abi.StepStats()
        rc = load().mfem_gpu_tri2d_step(self._h, C.byref(st))
        if raise_on_error:
            check(rc, "tri2d_step")
        elif rc in (abi.ERR_CUDA, abi.ERR_INVALID):
            check(rc, "tri2d_step")
        return st

    def get_state(self):
        x = np.zeros(2 * self.n_vertices)
        v = np.zeros(2 * self.n_vertices)
        s = np.zeros(3 * self.n_tris)
        R = np.zeros(4 * self.n_tris)
        la = np.zeros(3 * self.n_tris)
        check(load().mfem_gpu_tri2d_get_state(self._h, _p(x), _p(v), _p(s), _p(R), _p(la)),
              "tri2d_get_state")
        return dict(x=x.reshape(-1, 2), v=v.reshape(-1, 2), s=s.reshape(-1, 3),
                    R=R.reshape(-1, 4), la=la.reshape(-1, 3))

    def elem_update(self, x, h):
        nt = self.n_tris
        out = dict(R=np.zeros((nt, 4)), S=np.zeros((nt, 3)), dSdF=np.zeros((nt, 12)),
                   g=np.zeros((nt, 3)), H=np.zeros((nt, 9)), Hinv=np.zeros((nt, 9)),
                   Aloc=np.zeros((nt, 36)), gl=np.zeros((nt, 3)))
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        check(load().mfem_gpu_tri2d_elem_update(self._h, _p(x), h, *(_p(out[k]) for k in
                                                ("R", "S", "dSdF", "g", "H", "Hinv", "Aloc", "gl"))),
              "tri2d_elem_update")
        return out

    def get_system(self):
        rp = np.zeros(self.n_free + 1, dtype=np.int32)
        col = np.zeros(self.nnzb, dtype=np.int32)
        val = np.zeros(4 * self.nnzb)
        rhs = np.zeros(2 * self.n_free)
        check(load().mfem_gpu_tri2d_get_system(self._h, rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip),
                                               _p(val), _p(rhs)), "tri2d_get_system")
        return rp, col, val.reshape(-1, 2, 2), rhs

    def set_profiling(self, enable):
        check(load().mfem_gpu_tri2d_set_profiling(self._h, int(bool(enable))), "tri2d_set_profiling")

    def kernel_stats(self):
        """{kernel name: (total ms with profiling on, launches)}."""
        out = {}
        for k, name in enumerate(KERNELS):
            ms, n = C.c_double(), C.c_int64()
            check(load().mfem_gpu_tri2d_kernel_stats(self._h, k, C.byref(ms), C.byref(n)),
                  "tri2d_kernel_stats")
            out[name] = (ms.value, n.value)
        return out
