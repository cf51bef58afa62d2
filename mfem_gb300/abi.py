"""ctypes mirror of include/mfem_gb300.h (the C ABI of the GPU library).

The structs and enums here are byte-for-byte the ones declared in the header;
tests check the layout against the compiled library.
"""
import ctypes as C

ABI_VERSION = 1

# status codes
OK = 0
ERR_INVALID = 1
ERR_OOM = 2
ERR_CUDA = 3
ERR_NONFINITE = 4
ERR_CG_MAXITER = 5
ERR_LS_FAILED = 6
ERR_PROCRUSTES = 7
ERR_TIMEOUT = 8
ERR_NO_DEVICE = 9
ERR_UNSUPPORTED = 10
ERR_CAPACITY = 11

STATUS_NAMES = {
    OK: "ok", ERR_INVALID: "invalid argument", ERR_OOM: "out of device memory",
    ERR_CUDA: "CUDA error", ERR_NONFINITE: "non-finite value",
    ERR_CG_MAXITER: "PCG reached max iterations",
    ERR_LS_FAILED: "line search reached max iterations",
    ERR_PROCRUSTES: "singular rotation Hessian", ERR_TIMEOUT: "bounded wait timed out",
    ERR_NO_DEVICE: "no CUDA device", ERR_UNSUPPORTED: "unsupported option",
    ERR_CAPACITY: "capacity exceeded",
}

# MaterialModelType (reference src/config.h:61-68) and factory names
MATERIAL_SNH, MATERIAL_NH, MATERIAL_COROT, MATERIAL_FCR, MATERIAL_ARAP, MATERIAL_FUNG = range(6)

# LinearSolverType (reference src/config.h:45-59)
SOLVER_EIGEN_LLT = 0
SOLVER_EIGEN_LDLT = 1
SOLVER_EIGEN_LU = 2
SOLVER_CHOLMOD = 3
SOLVER_EIGEN_CG_DIAG = 5
SOLVER_EIGEN_CG_IC = 6
SOLVER_MINRES_ID = 8
SOLVER_MINRES_ADMM = 9
SOLVER_ADMM = 10
SOLVER_GPU_PCG_BLOCK = 100

# the elastic variable: MixedStretch ("mixed-stretch") or Stretch ("stretch")
FORMULATION_MIXED_STRETCH = 0
FORMULATION_STRETCH = 1

# BCScriptType (reference src/config.h:70-87) + additions
BC_NULL, BC_SCALEF, BC_HANG, BC_HANGENDS, BC_STRETCH = 0, 1, 2, 3, 4
BC_BEND, BC_TWIST, BC_ONEPOINT, BC_RANDOM = 7, 8, 13, 14
BC_PINMIN, BC_COMPRESS = 16, 17

PRECISION_FP64 = 0
PRECISION_MIXED = 1

PCG_KERNEL_PERSISTENT = 0
PCG_KERNEL_SPLIT = 1
PCG_KERNEL_FUSED = 2
PCG_KERNEL_AUTO = 3

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32),
        ("n_tets", C.c_int32),
        ("V_rest", _dp),
        ("V_init", _dp),
        ("v_init", _dp),
        ("tets", _ip),
        ("mu", _dp),
        ("lam", _dp),
        ("material", _ip),
        ("density", _dp),
        ("density_const", C.c_double),
        ("is_fixed", _ip),
        ("bc_type", C.c_int32),
        ("bc_axis", C.c_int32),
        ("bc_ratio", C.c_double),
        ("bc_velocity", C.c_double),
        ("dt", C.c_double),
        ("body_force", C.c_double * 3),
        ("bdf_order", C.c_int32),
        ("max_newton_iterations", C.c_int32),
        ("max_linesearch_iterations", C.c_int32),
        ("max_iterative_solver_iters", C.c_int32),
        ("iterative_solver_tolerance", C.c_double),
        ("newton_tol", C.c_double),
        ("newton_residual_tolerance", C.c_double),
        ("linear_solver", C.c_int32),
        ("precision", C.c_int32),
        ("pcg_kernel", C.c_int32),
        ("formulation", C.c_int32),
        ("reserved", C.c_int32 * 6),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("newton_iterations", C.c_int32),
        ("cg_iterations", C.c_int32),
        ("ls_iterations", C.c_int32),
        ("energy", C.c_double),
        ("energy_residual", C.c_double),
        ("decrement", C.c_double),
        ("alpha", C.c_double),
        ("residual0", C.c_double),
        ("residual", C.c_double),
        ("cg_error", C.c_double),
        ("device_ms", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Tri2dDesc(C.Structure):
    """mfem_tri2d_desc: a triangle mesh in the plane (the DIM = 2 path)."""
    _fields_ = [
        ("n_vertices", C.c_int32),
        ("n_tris", C.c_int32),
        ("V_rest", _dp),
        ("V_init", _dp),
        ("v_init", _dp),
        ("tris", _ip),
        ("mu", _dp),
        ("lam", _dp),
        ("material", _ip),
        ("density", _dp),
        ("density_const", C.c_double),
        ("is_fixed", _ip),
        ("bc_type", C.c_int32),
        ("bc_axis", C.c_int32),
        ("bc_ratio", C.c_double),
        ("bc_velocity", C.c_double),
        ("dt", C.c_double),
        ("body_force", C.c_double * 2),
        ("bdf_order", C.c_int32),
        ("max_newton_iterations", C.c_int32),
        ("max_linesearch_iterations", C.c_int32),
        ("max_iterative_solver_iters", C.c_int32),
        ("iterative_solver_tolerance", C.c_double),
        ("newton_tol", C.c_double),
        ("newton_residual_tolerance", C.c_double),
        ("linear_solver", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]
