"""Scenes and batches on the GPU, through the C ABI of libmfem_gb300.so."""
import ctypes as C

import numpy as np

from . import abi
from ._lib import check, load
from .desc import SceneSpec, make_desc

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def device_info():
    name = C.create_string_buffer(256)
    sms = C.c_int32(0)
    check(load().mfem_gpu_device_info(name, 256, C.byref(sms)), "device_info")
    return name.value.decode(), sms.value


def footprint(spec: SceneSpec) -> int:
    d = make_desc(spec)
    b = C.c_int64(0)
    check(load().mfem_gpu_scene_footprint(C.addressof(d.struct), C.byref(b)), "footprint")
    return b.value


class Scene:
    """One resident simulation instance (NewtonOptimizer<3> + its SimState)."""

    def __init__(self, spec: SceneSpec):
        L = load()
        self.spec = spec
        self._desc = make_desc(spec)
        h = C.c_void_p()
        check(L.mfem_gpu_scene_create(C.addressof(self._desc.struct), C.byref(h)), "scene_create")
        self._h = h
        nv, nt, nf = C.c_int32(), C.c_int32(), C.c_int32()
        L.mfem_gpu_scene_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(nf))
        self.n_vertices, self.n_tets, self.n_free = nv.value, nt.value, nf.value
        nb = C.c_int32()
        L.mfem_gpu_scene_bcsr_sizes(self._h, None, C.byref(nb))
        self.nnzb = nb.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().mfem_gpu_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pinned(self):
        n = C.c_int32()
        check(load().mfem_gpu_scene_pinned(self._h, C.byref(n), None), "pinned")
        v = np.zeros(n.value, dtype=np.int32)
        check(load().mfem_gpu_scene_pinned(self._h, C.byref(n), v.ctypes.data_as(_ip)), "pinned")
        return v

    def set_pins(self, positions):
        p = np.ascontiguousarray(positions, dtype=np.float64).ravel()
        check(load().mfem_gpu_scene_set_pins(self._h, _p(p)), "set_pins")

    def solo_batch_handle(self):
        h = C.c_void_p()
        check(load().mfem_gpu_scene_solo_batch(self._h, C.byref(h)), "solo_batch")
        return h

    def step(self, raise_on_error=True):
        """One timestep; its stats (.status says how it ended).  With
        raise_on_error=False a numerical failure (non-finite state, singular
        rotation Hessian, ...) is left to the caller; a CUDA error, a timed
        out wait or an invalid call still raises."""
        st = abi.StepStats()
        rc = load().mfem_gpu_scene_step(self._h, C.byref(st))
        if rc != abi.OK and (raise_on_error or rc in (abi.ERR_CUDA, abi.ERR_TIMEOUT, abi.ERR_INVALID)):
            check(rc, "scene_step")
        return st

    def get_state(self):
        x = np.zeros(3 * self.n_vertices)
        v = np.zeros(3 * self.n_vertices)
        s = np.zeros(6 * self.n_tets)
        R = np.zeros(9 * self.n_tets)
        la = np.zeros(6 * self.n_tets)
        check(load().mfem_gpu_scene_get_state(self._h, _p(x), _p(v), _p(s), _p(R), _p(la)), "get_state")
        return dict(x=x.reshape(-1, 3), v=v.reshape(-1, 3), s=s.reshape(-1, 6),
                    R=R.reshape(-1, 9), la=la.reshape(-1, 6))

    def positions(self):
        """Vertex positions only (3 per vertex, FP64)."""
        x = np.zeros(3 * self.n_vertices)
        check(load().mfem_gpu_scene_get_state(self._h, _p(x), None, None, None, None), "get_state")
        return x.reshape(-1, 3)

    def set_state(self, x=None, v=None, s=None, R=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()
        x, v, s, R = f(x), f(v), f(s), f(R)
        check(load().mfem_gpu_scene_set_state(self._h, _p(x), _p(v), _p(s), _p(R)), "set_state")

    def snapshot(self):
        """The scene's state between steps as bytes (x, BDF history, s, R,
        pins); restores into a scene of the same mesh in either precision."""
        n = C.c_int64()
        check(load().mfem_gpu_scene_snapshot_bytes(self._h, C.byref(n)), "snapshot_bytes")
        buf = (C.c_char * n.value)()
        check(load().mfem_gpu_scene_snapshot(self._h, buf, n.value), "snapshot")
        return bytes(buf)

    def restore(self, snap):
        buf = C.create_string_buffer(bytes(snap), len(snap))
        check(load().mfem_gpu_scene_restore(self._h, buf, len(snap)), "restore")

    def checkpoint(self):
        """Device-resident copy of the state; rollback() returns to it."""
        check(load().mfem_gpu_scene_checkpoint(self._h), "checkpoint")

    def rollback(self):
        check(load().mfem_gpu_scene_rollback(self._h), "rollback")

    def elem_update(self, x, h):
        nt = self.n_tets
        out = dict(R=np.zeros((nt, 9)), S=np.zeros((nt, 6)), dSdF=np.zeros((nt, 54)),
                   g=np.zeros((nt, 6)), H=np.zeros((nt, 36)), Hinv=np.zeros((nt, 36)),
                   Aloc=np.zeros((nt, 144)), gl=np.zeros((nt, 6)))
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        check(load().mfem_gpu_scene_elem_update(self._h, _p(x), h, *(_p(out[k]) for k in
              ("R", "S", "dSdF", "g", "H", "Hinv", "Aloc", "gl"))), "elem_update")
        return out

    def get_system(self):
        rp = np.zeros(self.n_free + 1, dtype=np.int32)
        col = np.zeros(self.nnzb, dtype=np.int32)
        val = np.zeros(9 * self.nnzb)
        rhs = np.zeros(3 * self.n_free)
        check(load().mfem_gpu_scene_get_system(self._h, rp.ctypes.data_as(_ip), col.ctypes.data_as(_ip),
                                               _p(val), _p(rhs)), "get_system")
        return rp, col, val.reshape(-1, 3, 3), rhs

    def pcg(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = C.c_int32()
        err = C.c_double()
        rc = load().mfem_gpu_scene_pcg(self._h, _p(b), _p(x), C.byref(it), C.byref(err))
        if rc not in (abi.OK, abi.ERR_CG_MAXITER):
            check(rc, "pcg")
        return x, it.value, err.value


KERNELS = ["k_elem_update", "k_assemble", "k_cg_init", "k_cg_spmv", "k_cg_update",
           "k_local_solve", "k_ls_energy", "k_apply", "k_step_begin", "k_step_end",
           "k_scalars_begin", "k_cg_solve", "k_cgf_iter", "k_cg_replace", "k_mr_init", "k_mr_elem",
           "k_mr_vert", "k_mr_update", "k_mr_export", "k_cg_loop"]


def set_profiling(batch_handle, enable=True):
    check(load().mfem_gpu_batch_set_profiling(batch_handle, int(enable)), "set_profiling")


def set_pcg_shape(batch_handle, stages, keep=0, unroll=1, pdl=0):
    """Shape of the batch's fused PCG iteration (mfem_gpu_batch_set_pcg_shape)."""
    check(load().mfem_gpu_batch_set_pcg_shape(batch_handle, int(stages), int(keep), int(unroll), int(pdl)),
          "set_pcg_shape")


def get_pcg_shape(batch_handle):
    v = [C.c_int32() for _ in range(4)]
    check(load().mfem_gpu_batch_get_pcg_shape(batch_handle, *(C.byref(x) for x in v)), "get_pcg_shape")
    return tuple(x.value for x in v)


def set_variants(batch_handle, elem_update=0, local_solve=0, ls_energy=0):
    """Register-budget variants of K1, K5, K6 by hand (0: built-in default)."""
    check(load().mfem_gpu_batch_set_variants(batch_handle, int(elem_update), int(local_solve), int(ls_energy)),
          "set_variants")


def tune_report(batch_handle):
    """The autotuner's record for the batch (dict)."""
    import json
    buf = C.create_string_buffer(1 << 16)
    check(load().mfem_gpu_batch_tune_report(batch_handle, buf, len(buf)), "tune_report")
    return json.loads(buf.value.decode())


def kernel_stats(batch_handle):
    """{kernel name: (total device ms, launches)} since profiling was enabled."""
    out = {}
    for k, name in enumerate(KERNELS):
        ms = C.c_double()
        n = C.c_int64()
        check(load().mfem_gpu_batch_kernel_stats(batch_handle, k, C.byref(ms), C.byref(n)), "kernel_stats")
        out[name] = (ms.value, n.value)
    return out


class Batch:
    """Independent scenes stepped together: one launch per kernel phase."""

    def __init__(self, scenes):
        self.scenes = list(scenes)
        arr = (C.c_void_p * len(self.scenes))(*[s.handle.value for s in self.scenes])
        h = C.c_void_p()
        check(load().mfem_gpu_batch_create(arr, len(self.scenes), C.byref(h)), "batch_create")
        self._h = h
        self._stats = (abi.StepStats * len(self.scenes))()

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().mfem_gpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def step(self, raise_on_error=True):
        """One timestep of every scene; per-scene stats (their .status says
        how each scene's step ended).  With raise_on_error=False a scene's
        numerical failure is left to the caller (the batch itself stays
        usable); a CUDA error still raises."""
        rc = load().mfem_gpu_batch_step(self._h, self._stats)
        if rc != abi.OK and (raise_on_error or rc in (abi.ERR_CUDA, abi.ERR_TIMEOUT, abi.ERR_INVALID)):
            check(rc, "batch_step")
        return [abi.StepStats.from_buffer_copy(st) for st in self._stats]

    def step_n(self, steps, raise_on_error=True):
        """`steps` timesteps of every scene, each scene at its own pace
        (mfem_gpu_batch_step_n).  Returns (stats per scene, summed over its
        steps; step_done_ms: scenes x steps device times from the call's
        start at which each step was done)."""
        done = np.zeros((len(self.scenes), max(int(steps), 1)))
        rc = load().mfem_gpu_batch_step_n(self._h, int(steps), self._stats, done.ctypes.data_as(_dp))
        if rc != abi.OK and (raise_on_error or rc in (abi.ERR_CUDA, abi.ERR_TIMEOUT, abi.ERR_INVALID)):
            check(rc, "batch_step_n")
        return [abi.StepStats.from_buffer_copy(st) for st in self._stats], done


def set_tuning(mode):
    """Autotuner mode for batches created from now on (mfem_gpu_set_tuning:
    0 defaults, 1 time on a cache miss, 2 always, -1 the environment's)."""
    check(load().mfem_gpu_set_tuning(int(mode)), "set_tuning")


def set_priority(batch_handle, priority):
    """Stream priority of a batch against other batches (0 default, higher
    runs first; mfem_gpu_batch_set_priority)."""
    check(load().mfem_gpu_batch_set_priority(batch_handle, int(priority)), "set_priority")


def lane_partition(weights, lanes):
    """Indices per lane: longest-processing-time first by weight (a scene's
    tets), each to the least-loaded lane; empty lanes dropped."""
    out = [[] for _ in range(max(1, int(lanes)))]
    load_ = [0.0] * len(out)
    for i in sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i)):
        k = min(range(len(out)), key=lambda j: (load_[j], j))
        out[k].append(i)
        load_[k] += float(weights[i])
    return [sorted(l) for l in out if l]


class Lanes:
    """Scenes split into `lanes` batches (balanced by tets) that step side by
    side, each on its own stream and host thread (mfem_gpu_batches_step_n):
    a latency-bound small scene waits only for its own batch's launches.
    The lane of the smallest scenes on average runs at the highest stream
    priority.  A scene's arithmetic does not depend on its batch, so every
    result is the one of the same scene in a single batch of the same PCG
    form."""

    def __init__(self, scenes, lanes=4):
        self.scenes = list(scenes)
        self.parts = lane_partition([s.n_tets for s in self.scenes], lanes)
        self.batches = [Batch([self.scenes[i] for i in p]) for p in self.parts]
        mean = [np.mean([self.scenes[i].n_tets for i in p]) for p in self.parts]
        for r, k in enumerate(np.argsort(mean)):
            set_priority(self.batches[k].handle, max(0, len(self.parts) - 1 - r))
        self._order = [i for p in self.parts for i in p]
        self._stats = (abi.StepStats * len(self.scenes))()

    def close(self):
        for b in self.batches:
            b.close()
        self.batches = []

    def step(self, raise_on_error=True):
        """One timestep of every scene (each lane one mfem_gpu_batch_step)."""
        out = [None] * len(self.scenes)
        for p, b in zip(self.parts, self.batches):
            for i, st in zip(p, b.step(raise_on_error=raise_on_error)):
                out[i] = st
        return out

    def step_n(self, steps, raise_on_error=True):
        """`steps` timesteps of every scene, each at its own pace, the lanes
        concurrently; (stats per scene in the scenes' order, step_done_ms
        scenes x steps from each lane's start)."""
        n = len(self.scenes)
        done = np.zeros((n, max(int(steps), 1)))
        arr = (C.c_void_p * len(self.batches))(*[b.handle.value for b in self.batches])
        rc = load().mfem_gpu_batches_step_n(arr, len(self.batches), int(steps), self._stats,
                                             done.ctypes.data_as(_dp))
        if rc != abi.OK and (raise_on_error or rc in (abi.ERR_CUDA, abi.ERR_TIMEOUT, abi.ERR_INVALID)):
            check(rc, "batches_step_n")
        stats = [None] * n
        out_done = np.zeros_like(done)
        for pos, i in enumerate(self._order):
            stats[i] = abi.StepStats.from_buffer_copy(self._stats[pos])
            out_done[i] = done[pos]
        return stats, out_done
