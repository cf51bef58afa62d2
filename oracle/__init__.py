"""TEST INFRASTRUCTURE ONLY: ctypes loader for the FP64 CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
import this package, to check results or as the timed CPU baseline.  See
mfem_oracle.h for what the oracle restates and how far parity is pinned.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmfem_oracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def build(force=False):
    """Compiles the oracle with the Makefile beside this file."""
    srcs = [os.path.join(_HERE, f) for f in ("mfem_oracle.cpp", "mfem_oracle2d.cpp",
                                             "mfem_oracle.h", "Makefile",
                                             os.path.join("..", "include", "mfem_gb300.h"))]
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(s) for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_procrustes.argtypes = [_dp, _dp, _dp, C.c_int, _dp, C.c_double, C.c_int, _ip]
        L.oracle_dsvd_dRdF.argtypes = [_dp, _dp]
        L.oracle_polar.argtypes = [_dp, _dp, C.c_int, _dp, _dp]
        L.oracle_material_energy.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.oracle_material_energy.restype = C.c_double
        L.oracle_material_gradient.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp]
        L.oracle_material_hessian.argtypes = [C.c_int, C.c_double, C.c_double, _dp, C.c_int, _dp]
        L.oracle_psd_fix.argtypes = [_dp, C.c_int, C.c_double]
        L.oracle_material9.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_int]
        L.oracle_material9.restype = C.c_double
        L.oracle_scene_create.argtypes = [C.c_void_p, _ip]
        L.oracle_scene_create.restype = C.c_void_p
        L.oracle_scene_destroy.argtypes = [C.c_void_p]
        L.oracle_scene_step.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_scene_sizes.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
        L.oracle_scene_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.oracle_scene_set_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.oracle_scene_set_positions.argtypes = [C.c_void_p, _dp]
        L.oracle_scene_elem_update.argtypes = [C.c_void_p, _dp, C.c_double] + [_dp] * 8
        L.oracle_scene_get_system.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
        L.oracle_scene_energy.argtypes = [C.c_void_p, C.c_double]
        L.oracle_scene_energy.restype = C.c_double
        L.oracle_scene_pcg.argtypes = [C.c_void_p, _dp, _dp, _ip, _dp]
        L.oracle_scene_kkt_size.argtypes = [C.c_void_p]
        L.oracle_scene_kkt_rhs.argtypes = [C.c_void_p, _dp]
        L.oracle_scene_kkt_mul.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_scene_minres.argtypes = [C.c_void_p, _dp, _dp, _ip, _dp]
        L.oracle_scene_schur_solve.argtypes = [C.c_void_p, _dp, _ip, _dp]
        L.oracle_scene_update_system.argtypes = [C.c_void_p]
        L.oracle2d_polar.argtypes = [_dp, _dp, _dp, _dp]
        L.oracle2d_svd.argtypes = [_dp, _dp, _dp, _dp]
        L.oracle2d_material.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, C.c_int]
        L.oracle2d_material.restype = C.c_double
        L.oracle2d_create.argtypes = [C.c_void_p, _ip]
        L.oracle2d_create.restype = C.c_void_p
        L.oracle2d_destroy.argtypes = [C.c_void_p]
        L.oracle2d_step.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle2d_sizes.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
        L.oracle2d_get_state.argtypes = [C.c_void_p] + [_dp] * 5
        L.oracle2d_elem_update.argtypes = [C.c_void_p, _dp, C.c_double] + [_dp] * 8
        L.oracle2d_get_system.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
        L.oracle2d_energy.argtypes = [C.c_void_p, C.c_double]
        L.oracle2d_energy.restype = C.c_double
        L.oracle2d_direction.argtypes = [C.c_void_p, _dp, _dp, _dp, _ip]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def set_threads(n):
    return lib().oracle_set_threads(int(n))


def procrustes(R0, A, B, compute_gradients=True, tol=1e-6, max_iter=100):
    """newton_procrustes on 3x3 numpy matrices; returns (R, dRdF 9x9, iters)."""
    R = np.asfortranarray(R0, dtype=np.float64).copy(order="F")
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    d = np.zeros((9, 9), order="F")
    it = C.c_int32(0)
    st = lib().oracle_procrustes(_p(R), _p(A), _p(B), int(compute_gradients), _p(d),
                                 tol, max_iter, C.byref(it))
    if st != 0:
        raise RuntimeError(f"procrustes status {st}")
    return R, d, it.value


def dsvd_dRdF(F):
    F = np.asfortranarray(F, dtype=np.float64)
    d = np.zeros((9, 9), order="F")
    lib().oracle_dsvd_dRdF(_p(F), _p(d))
    return d


def polar(F, R0=None, compute_gradients=True):
    R = np.eye(3, order="F") if R0 is None else np.asfortranarray(R0, dtype=np.float64).copy(order="F")
    F = np.asfortranarray(F, dtype=np.float64)
    s = np.zeros(6)
    dsdF = np.zeros((6, 9), order="F")
    st = lib().oracle_polar(_p(R), _p(F), int(compute_gradients), _p(s), _p(dsdF))
    if st != 0:
        raise RuntimeError(f"polar status {st}")
    return R, s, dsdF


def material_energy(mtype, mu, lam, s):
    s = np.ascontiguousarray(s, dtype=np.float64)
    return lib().oracle_material_energy(mtype, mu, lam, _p(s))


def material_gradient(mtype, mu, lam, s):
    s = np.ascontiguousarray(s, dtype=np.float64)
    g = np.zeros(6)
    lib().oracle_material_gradient(mtype, mu, lam, _p(s), _p(g))
    return g


def material_hessian(mtype, mu, lam, s, psd_fix=True):
    s = np.ascontiguousarray(s, dtype=np.float64)
    H = np.zeros((6, 6), order="F")
    lib().oracle_material_hessian(mtype, mu, lam, _p(s), int(psd_fix), _p(H))
    return H


def material9(mtype, mu, lam, F, psd_fix=True):
    """psi, dpsi/dF (9) and d2psi/dF2 (9x9) on the column-major flattened F
    (the standard-FEM variable's Vector9d forms)."""
    f = np.asfortranarray(F, dtype=np.float64).ravel(order="F").copy()
    g = np.zeros(9)
    H = np.zeros((9, 9), order="F")
    psi = lib().oracle_material9(mtype, mu, lam, _p(f), _p(g), _p(H), int(psd_fix))
    return psi, g, H


def psd_fix(H, tol=1e-6):
    H = np.asfortranarray(H, dtype=np.float64).copy(order="F")
    lib().oracle_psd_fix(_p(H), H.shape[0], tol)
    return H


class OracleScene:
    """FP64 CPU scene with the same descriptor as the GPU library."""

    def __init__(self, spec):
        from mfem_gb300.desc import make_desc
        self._desc = make_desc(spec)
        st = C.c_int32(0)
        self._h = lib().oracle_scene_create(C.addressof(self._desc.struct), C.byref(st))
        if not self._h:
            raise RuntimeError(f"oracle scene create failed: status {st.value}")
        self.create_status = st.value
        nv, nt, nf, nb = (C.c_int32() for _ in range(4))
        lib().oracle_scene_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(nf), C.byref(nb))
        self.n_vertices, self.n_tets, self.n_free, self.nnzb = nv.value, nt.value, nf.value, nb.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_scene_destroy(h)
            self._h = None

    def step(self):
        from mfem_gb300.abi import StepStats
        st = StepStats()
        lib().oracle_scene_step(self._h, C.byref(st))
        return st

    def get_state(self):
        x = np.zeros(3 * self.n_vertices)
        v = np.zeros(3 * self.n_vertices)
        s = np.zeros(6 * self.n_tets)
        R = np.zeros(9 * self.n_tets)
        la = np.zeros(6 * self.n_tets)
        lib().oracle_scene_get_state(self._h, _p(x), _p(v), _p(s), _p(R), _p(la))
        return dict(x=x.reshape(-1, 3), v=v.reshape(-1, 3), s=s.reshape(-1, 6),
                    R=R.reshape(-1, 9), la=la.reshape(-1, 6))

    def set_state(self, x=None, v=None, s=None, R=None, la=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()
        x, v, s, R, la = f(x), f(v), f(s), f(R), f(la)
        lib().oracle_scene_set_state(self._h, _p(x), _p(v), _p(s), _p(R), _p(la))

    def set_positions(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        lib().oracle_scene_set_positions(self._h, _p(x))

    def elem_update(self, x, h):
        nt = self.n_tets
        out = dict(R=np.zeros((nt, 9)), S=np.zeros((nt, 6)), dSdF=np.zeros((nt, 54)),
                   g=np.zeros((nt, 6)), H=np.zeros((nt, 36)), Hinv=np.zeros((nt, 36)),
                   Aloc=np.zeros((nt, 144)), gl=np.zeros((nt, 6)))
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        lib().oracle_scene_elem_update(self._h, _p(x), h, *(_p(out[k]) for k in
                                       ("R", "S", "dSdF", "g", "H", "Hinv", "Aloc", "gl")))
        return out

    def get_system(self):
        rp = np.zeros(self.n_free + 1, dtype=np.int32)
        col = np.zeros(self.nnzb, dtype=np.int32)
        val = np.zeros(9 * self.nnzb)
        rhs = np.zeros(3 * self.n_free)
        lib().oracle_scene_get_system(self._h, rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip),
                                      _p(val), _p(rhs))
        return rp, col, val.reshape(-1, 3, 3), rhs

    def energy(self, alpha):
        return lib().oracle_scene_energy(self._h, alpha)

    def pcg(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = C.c_int32()
        err = C.c_double()
        lib().oracle_scene_pcg(self._h, _p(b), _p(x), C.byref(it), C.byref(err))
        return x, it.value, err.value

    # ---- the (x, s, lambda) system of "minres-indefinite-block" ----------
    # at the state of the last update_system(): KKT vectors are
    # [x: 3 n_free][s: 6 n_tets][lambda: 6 n_tets]
    def update_system(self):
        return lib().oracle_scene_update_system(self._h)

    def kkt_rhs(self):
        r = np.zeros(lib().oracle_scene_kkt_size(self._h))
        lib().oracle_scene_kkt_rhs(self._h, _p(r))
        return r

    def kkt_mul(self, w):
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros_like(w)
        lib().oracle_scene_kkt_mul(self._h, _p(w), _p(out))
        return out

    def minres(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = C.c_int32()
        err = C.c_double()
        st = lib().oracle_scene_minres(self._h, _p(b), _p(x), C.byref(it), C.byref(err))
        return x, it.value, err.value, st

    def schur_solve(self):
        """PCG on the Schur system then the local solve: [dx; ds; lambda]."""
        x = np.zeros(lib().oracle_scene_kkt_size(self._h))
        it = C.c_int32()
        err = C.c_double()
        lib().oracle_scene_schur_solve(self._h, _p(x), C.byref(it), C.byref(err))
        return x, it.value, err.value


# ---- the 2-D path (mfem_oracle2d.cpp) --------------------------------------

def polar2(F, compute_gradients=True):
    """polar_svd<2>: (R 2x2, s[3], ds/dF 3x4 on the column-major vec(F), status)."""
    F = np.asfortranarray(F, dtype=np.float64)
    R = np.zeros((2, 2), order="F")
    s = np.zeros(3)
    dsdF = np.zeros((3, 4), order="F")
    st = lib().oracle2d_polar(_p(R), _p(F), _p(s), _p(dsdF) if compute_gradients else None)
    return R, s, dsdF, st


def svd2(F):
    F = np.asfortranarray(F, dtype=np.float64)
    sig = np.zeros(2)
    U = np.zeros((2, 2), order="F")
    V = np.zeros((2, 2), order="F")
    lib().oracle2d_svd(_p(F), _p(sig), _p(U), _p(V))
    return sig, U, V


def material2(mtype, mu, lam, s, psd_fix=True):
    """psi, gradient (3) and Hessian (3x3) of a 3-vector material."""
    s = np.ascontiguousarray(s, dtype=np.float64)
    g = np.zeros(3)
    H = np.zeros((3, 3), order="F")
    psi = lib().oracle2d_material(mtype, mu, lam, _p(s), _p(g), _p(H), int(psd_fix))
    return psi, g, H


class OracleTri2d:
    """FP64 CPU 2-D scene with the same descriptor as the GPU library."""

    def __init__(self, spec):
        from mfem_gb300.desc import make_tri2d_desc
        self._desc = make_tri2d_desc(spec)
        st = C.c_int32(0)
        self._h = lib().oracle2d_create(C.addressof(self._desc.struct), C.byref(st))
        self.create_status = st.value
        if not self._h:
            raise RuntimeError(f"oracle 2-D scene create failed: status {st.value}")
        nv, nt, nf, nb = (C.c_int32() for _ in range(4))
        lib().oracle2d_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(nf), C.byref(nb))
        self.n_vertices, self.n_tris, self.n_free, self.nnzb = nv.value, nt.value, nf.value, nb.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle2d_destroy(h)
            self._h = None

    def step(self):
        from mfem_gb300.abi import StepStats
        st = StepStats()
        lib().oracle2d_step(self._h, C.byref(st))
        return st

    def get_state(self):
        x = np.zeros(2 * self.n_vertices)
        v = np.zeros(2 * self.n_vertices)
        s = np.zeros(3 * self.n_tris)
        R = np.zeros(4 * self.n_tris)
        la = np.zeros(3 * self.n_tris)
        lib().oracle2d_get_state(self._h, _p(x), _p(v), _p(s), _p(R), _p(la))
        return dict(x=x.reshape(-1, 2), v=v.reshape(-1, 2), s=s.reshape(-1, 3),
                    R=R.reshape(-1, 4), la=la.reshape(-1, 3))

    def elem_update(self, x, h):
        nt = self.n_tris
        out = dict(R=np.zeros((nt, 4)), S=np.zeros((nt, 3)), dSdF=np.zeros((nt, 12)),
                   g=np.zeros((nt, 3)), H=np.zeros((nt, 9)), Hinv=np.zeros((nt, 9)),
                   Aloc=np.zeros((nt, 36)), gl=np.zeros((nt, 3)))
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        lib().oracle2d_elem_update(self._h, _p(x), h, *(_p(out[k]) for k in
                                   ("R", "S", "dSdF", "g", "H", "Hinv", "Aloc", "gl")))
        return out

    def get_system(self):
        rp = np.zeros(self.n_free + 1, dtype=np.int32)
        col = np.zeros(self.nnzb, dtype=np.int32)
        val = np.zeros(4 * self.nnzb)
        rhs = np.zeros(2 * self.n_free)
        lib().oracle2d_get_system(self._h, rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip),
                                  _p(val), _p(rhs))
        return rp, col, val.reshape(-1, 2, 2), rhs

    def energy(self, alpha):
        return lib().oracle2d_energy(self._h, alpha)

    def direction(self):
        """(dx per vertex, ds, lambda, PCG iterations) of one Newton
        iteration at the current state, without stepping."""
        dx = np.zeros(2 * self.n_vertices)
        ds = np.zeros(3 * self.n_tris)
        la = np.zeros(3 * self.n_tris)
        it = C.c_int32()
        lib().oracle2d_direction(self._h, _p(dx), _p(ds), _p(la), C.byref(it))
        return dx.reshape(-1, 2), ds.reshape(-1, 3), la.reshape(-1, 3), it.value
