"""Loads libmfem_gb300.so (the CUDA library) and declares its C ABI.

There is no CPU fallback: if the library is missing or no GPU is visible,
the calls fail with an error.
"""
import ctypes as C
import os
import re

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmfem_gb300.so")
HEADER = os.path.join(_HERE, "..", "include", "mfem_gb300.h")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_vp = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "mfem_gpu_abi_version": (C.c_int, []),
    "mfem_gpu_set_device": (C.c_int, [C.c_int]),
    "mfem_gpu_device_info": (C.c_int, [C.c_char_p, C.c_int, _ip]),
    "mfem_gpu_selftest_bounded_wait": (C.c_int, [_dp]),
    "mfem_gpu_status_string": (C.c_char_p, [C.c_int]),
    "mfem_gpu_scene_create": (C.c_int, [_vp, C.POINTER(_vp)]),
    "mfem_gpu_scene_destroy": (C.c_int, [_vp]),
    "mfem_gpu_scene_step": (C.c_int, [_vp, _vp]),
    "mfem_gpu_scene_footprint": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "mfem_gpu_scene_sizes": (C.c_int, [_vp, _ip, _ip, _ip]),
    "mfem_gpu_scene_get_state": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "mfem_gpu_scene_set_state": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "mfem_gpu_scene_snapshot_bytes": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "mfem_gpu_scene_snapshot": (C.c_int, [_vp, _vp, C.c_int64]),
    "mfem_gpu_scene_restore": (C.c_int, [_vp, _vp, C.c_int64]),
    "mfem_gpu_scene_checkpoint": (C.c_int, [_vp]),
    "mfem_gpu_scene_rollback": (C.c_int, [_vp]),
    "mfem_gpu_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int32, C.POINTER(_vp)]),
    "mfem_gpu_batch_destroy": (C.c_int, [_vp]),
    "mfem_gpu_batch_step": (C.c_int, [_vp, _vp]),
    "mfem_gpu_batch_step_n": (C.c_int, [_vp, C.c_int32, _vp, _dp]),
    "mfem_gpu_batches_step_n": (C.c_int, [C.POINTER(_vp), C.c_int32, C.c_int32, _vp, _dp]),
    "mfem_gpu_scene_elem_update": (C.c_int, [_vp, _dp, C.c_double] + [_dp] * 8),
    "mfem_gpu_scene_bcsr_sizes": (C.c_int, [_vp, _ip, _ip]),
    "mfem_gpu_scene_get_system": (C.c_int, [_vp, _ip, _ip, _dp, _dp]),
    "mfem_gpu_scene_pcg": (C.c_int, [_vp, _dp, _dp, _ip, _dp]),
    "mfem_gpu_scene_pinned": (C.c_int, [_vp, _ip, _ip]),
    "mfem_gpu_scene_set_pins": (C.c_int, [_vp, _dp]),
    "mfem_gpu_scene_solo_batch": (C.c_int, [_vp, C.POINTER(_vp)]),
    "mfem_gpu_batch_set_profiling": (C.c_int, [_vp, C.c_int]),
    "mfem_gpu_batch_set_priority": (C.c_int, [_vp, C.c_int32]),
    "mfem_gpu_set_tuning": (C.c_int, [C.c_int32]),
    "mfem_gpu_batch_kernel_stats": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(C.c_int64)]),
    "mfem_gpu_batch_set_pcg_shape": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "mfem_gpu_batch_get_pcg_shape": (C.c_int, [_vp] + [C.POINTER(C.c_int32)] * 4),
    "mfem_gpu_batch_tune_report": (C.c_int, [_vp, C.c_char_p, C.c_int32]),
    "mfem_gpu_batch_set_variants": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32]),
    "mfem_gpu_kernel_name": (C.c_int, [C.c_int, C.c_char_p, C.c_int]),
    "mfem_gpu_bsr_pcg_noalloc": (C.c_int, [C.c_int32, C.c_int32, _vp, _vp, _vp, _vp, _vp, C.c_int32,
                                           C.c_double, _vp, _ip, _dp]),
    "mfem_gpu_tri2d_create": (C.c_int, [_vp, C.POINTER(_vp)]),
    "mfem_gpu_tri2d_destroy": (C.c_int, [_vp]),
    "mfem_gpu_tri2d_step": (C.c_int, [_vp, _vp]),
    "mfem_gpu_tri2d_sizes": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "mfem_gpu_tri2d_get_state": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "mfem_gpu_tri2d_elem_update": (C.c_int, [_vp, _dp, C.c_double] + [_dp] * 8),
    "mfem_gpu_tri2d_get_system": (C.c_int, [_vp, _ip, _ip, _dp, _dp]),
    "mfem_gpu_tri2d_set_profiling": (C.c_int, [_vp, C.c_int]),
    "mfem_gpu_tri2d_kernel_stats": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(C.c_int64)]),
}


def header_symbols():
    """Function names declared in include/mfem_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mfem_gpu_\w+)\s*\(", text)))


def load(path=None):
    """Returns the loaded library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from .build import build
        build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if L.mfem_gpu_abi_version() != abi.ABI_VERSION:
        raise RuntimeError("libmfem_gb300.so ABI version mismatch")
    _lib = L
    return L


class MfemError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = load().mfem_gpu_status_string(status).decode()
        super().__init__(f"{what}: status {status} ({msg})")


def check(status, what=""):
    if status != abi.OK:
        raise MfemError(status, what)
    return status
