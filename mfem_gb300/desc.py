"""Building an mfem_scene_desc (include/mfem_gb300.h) from numpy arrays.

`make_desc` returns the ctypes struct plus the arrays it points into (keep the
returned object alive while the struct is in use).
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi


@dataclass
class SceneSpec:
    """Host-side description of one simulation instance.

    Mirrors the fields the reference reads from a scene JSON
    (src/simulation_state.cpp:92-366) plus per-element material arrays.
    """
    V_rest: np.ndarray
    tets: np.ndarray
    mu: np.ndarray
    lam: np.ndarray
    V_init: np.ndarray = None
    v_init: np.ndarray = None
    material: np.ndarray = None
    density: np.ndarray = None
    density_const: float = 1000.0
    is_fixed: np.ndarray = None
    bc_type: int = abi.BC_NULL
    bc_axis: int = 0
    bc_ratio: float = 0.1
    bc_velocity: float = 0.1
    dt: float = 0.034
    body_force: tuple = (0.0, -9.8, 0.0)
    bdf_order: int = 1
    max_newton_iterations: int = 5
    max_linesearch_iterations: int = 20
    max_iterative_solver_iters: int = 500
    iterative_solver_tolerance: float = 1e-4
    newton_tol: float = 1e-10
    newton_residual_tolerance: float = 0.0
    linear_solver: int = abi.SOLVER_EIGEN_CG_DIAG
    precision: int = abi.PRECISION_FP64
    pcg_kernel: int = abi.PCG_KERNEL_PERSISTENT
    formulation: int = abi.FORMULATION_MIXED_STRETCH
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n_vertices(self):
        return int(self.V_rest.shape[0])

    @property
    def n_tets(self):
        return int(self.tets.shape[0])


class _Desc:
    def __init__(self, struct, keep):
        self.struct = struct
        self._keep = keep

    @property
    def ptr(self):
        return C.byref(self.struct)


def _f64(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _i32(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def make_desc(spec: SceneSpec) -> _Desc:
    nv, nt = spec.n_vertices, spec.n_tets
    keep = []

    def dp(a, n):
        if a is None:
            return C.cast(None, C.POINTER(C.c_double))
        arr = _f64(a, n)
        keep.append(arr)
        return arr.ctypes.data_as(C.POINTER(C.c_double))

    def ip(a, n):
        if a is None:
            return C.cast(None, C.POINTER(C.c_int32))
        arr = _i32(a, n)
        keep.append(arr)
        return arr.ctypes.data_as(C.POINTER(C.c_int32))

    d = abi.SceneDesc()
    d.n_vertices = nv
    d.n_tets = nt
    d.V_rest = dp(spec.V_rest, 3 * nv)
    d.V_init = dp(spec.V_init, 3 * nv)
    d.v_init = dp(spec.v_init, 3 * nv)
    d.tets = ip(spec.tets, 4 * nt)
    d.mu = dp(np.broadcast_to(np.asarray(spec.mu, np.float64), (nt,)), nt)
    d.lam = dp(np.broadcast_to(np.asarray(spec.lam, np.float64), (nt,)), nt)
    d.material = ip(None if spec.material is None
                    else np.broadcast_to(np.asarray(spec.material, np.int32), (nt,)), nt)
    d.density = dp(None if spec.density is None
                   else np.broadcast_to(np.asarray(spec.density, np.float64), (nt,)), nt)
    d.density_const = float(spec.density_const)
    d.is_fixed = ip(spec.is_fixed, nv)
    d.bc_type = int(spec.bc_type)
    d.bc_axis = int(spec.bc_axis)
    d.bc_ratio = float(spec.bc_ratio)
    d.bc_velocity = float(spec.bc_velocity)
    d.dt = float(spec.dt)
    for k in range(3):
        d.body_force[k] = float(spec.body_force[k])
    d.bdf_order = int(spec.bdf_order)
    d.max_newton_iterations = int(spec.max_newton_iterations)
    d.max_linesearch_iterations = int(spec.max_linesearch_iterations)
    d.max_iterative_solver_iters = int(spec.max_iterative_solver_iters)
    d.iterative_solver_tolerance = float(spec.iterative_solver_tolerance)
    d.newton_tol = float(spec.newton_tol)
    d.newton_residual_tolerance = float(spec.newton_residual_tolerance)
    d.linear_solver = int(spec.linear_solver)
    d.precision = int(spec.precision)
    d.pcg_kernel = int(spec.pcg_kernel)
    d.formulation = int(spec.formulation)
    return _Desc(d, keep)


@dataclass
class Tri2dSpec:
    """Host-side description of one 2-D (triangle mesh) instance: what
    SimState<2>::load reads (src/simulation_state.cpp:43-60, 92-366), with
    per-triangle material arrays.  Triangles are counter-clockwise."""
    V_rest: np.ndarray
    tris: np.ndarray
    mu: np.ndarray
    lam: np.ndarray
    V_init: np.ndarray = None
    v_init: np.ndarray = None
    material: np.ndarray = None
    density: np.ndarray = None
    density_const: float = 1000.0
    is_fixed: np.ndarray = None
    bc_type: int = abi.BC_NULL
    bc_axis: int = 0
    bc_ratio: float = 0.1
    bc_velocity: float = 0.1
    dt: float = 0.0333
    body_force: tuple = (0.0, -9.8)
    bdf_order: int = 1
    max_newton_iterations: int = 10
    max_linesearch_iterations: int = 20
    max_iterative_solver_iters: int = 500
    iterative_solver_tolerance: float = 1e-8
    newton_tol: float = 1e-10
    newton_residual_tolerance: float = 0.0
    linear_solver: int = abi.SOLVER_EIGEN_CG_DIAG
    name: str = ""

    @property
    def n_vertices(self):
        return int(self.V_rest.shape[0])

    @property
    def n_tris(self):
        return int(self.tris.shape[0])


def make_tri2d_desc(spec: Tri2dSpec) -> _Desc:
    nv, nt = spec.n_vertices, spec.n_tris
    keep = []

    def dp(a, n):
        if a is None:
            return C.cast(None, C.POINTER(C.c_double))
        arr = _f64(a, n)
        keep.append(arr)
        return arr.ctypes.data_as(C.POINTER(C.c_double))

    def ip(a, n):
        if a is None:
            return C.cast(None, C.POINTER(C.c_int32))
        arr = _i32(a, n)
        keep.append(arr)
        return arr.ctypes.data_as(C.POINTER(C.c_int32))

    d = abi.Tri2dDesc()
    d.n_vertices = nv
    d.n_tris = nt
    d.V_rest = dp(spec.V_rest, 2 * nv)
    d.V_init = dp(spec.V_init, 2 * nv)
    d.v_init = dp(spec.v_init, 2 * nv)
    d.tris = ip(spec.tris, 3 * nt)
    d.mu = dp(np.broadcast_to(np.asarray(spec.mu, np.float64), (nt,)), nt)
    d.lam = dp(np.broadcast_to(np.asarray(spec.lam, np.float64), (nt,)), nt)
    d.material = ip(None if spec.material is None
                    else np.broadcast_to(np.asarray(spec.material, np.int32), (nt,)), nt)
    d.density = dp(None if spec.density is None
                   else np.broadcast_to(np.asarray(spec.density, np.float64), (nt,)), nt)
    d.density_const = float(spec.density_const)
    d.is_fixed = ip(spec.is_fixed, nv)
    d.bc_type = int(spec.bc_type)
    d.bc_axis = int(spec.bc_axis)
    d.bc_ratio = float(spec.bc_ratio)
    d.bc_velocity = float(spec.bc_velocity)
    d.dt = float(spec.dt)
    for k in range(2):
        d.body_force[k] = float(spec.body_force[k])
    d.bdf_order = int(spec.bdf_order)
    d.max_newton_iterations = int(spec.max_newton_iterations)
    d.max_linesearch_iterations = int(spec.max_linesearch_iterations)
    d.max_iterative_solver_iters = int(spec.max_iterative_solver_iters)
    d.iterative_solver_tolerance = float(spec.iterative_solver_tolerance)
    d.newton_tol = float(spec.newton_tol)
    d.newton_residual_tolerance = float(spec.newton_residual_tolerance)
    d.linear_solver = int(spec.linear_solver)
    return _Desc(d, keep)
