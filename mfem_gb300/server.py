"""Serving loop: continuous batching of simulation instances on one GPU.

Requests (a SceneSpec and a number of timesteps) arrive over time.  The loop
admits them in arrival order while their device footprint
(mfem_gpu_scene_footprint) fits the memory budget, keeps every admitted
instance's state resident (positions, velocities, stretch variables,
rotations, BDF history and solver state live in the scene's device arena),
and at every tick steps ALL admitted instances of a precision together: one
batch, one launch per kernel phase for all of them.  The mixed-precision
and the FP64 group tick independently, each on its own stream and thread,
each starting its next tick as soon as its last one ends.  A tick takes up to
`steps_per_tick` timesteps of every instance with each instance at its own
pace (mfem_gpu_batch_step_n: an instance whose Newton loop ends starts its
next timestep at once instead of waiting for the slowest one), bounded by
the fewest timesteps any member still owes; with steps_per_tick = 1 every
tick is one mfem_gpu_batch_step.  An instance that has taken its timesteps
leaves the batch, its memory is freed and the next queued request takes its
place at the next tick, so requests that arrive while others are on the GPU
join them there.  Batches are created with the autotuner off
(mfem_gpu_set_tuning(0)) unless `tune` is set, so that membership changes
do not pay for timing runs.

Scenes are built on a worker thread (the host mesh build and the arena
upload), overlapping the GPU ticks.  A scene's arithmetic does not depend on
which other scenes share its batch (per-scene tiles and fixed-order
reductions), so every result is bitwise the one the request would get alone.

Precision escalation: before every tick each mixed-precision scene keeps a
device-resident checkpoint of its state (positions, BDF history, s, R,
pins; mfem_gpu_scene_checkpoint).  A mixed scene whose step ends with a
failed line search (every trial step rejected, MFEM_ERR_LS_FAILED), a
singular rotation Hessian (MFEM_ERR_PROCRUSTES) or a non-finite state has
reached what FP32 matrices and directions can resolve -- in very soft
bodies at large deformation the clamped Hessian eigenvalues (1e-6 h^2
against O(10)) are below FP32 rounding, and later steps diverge.  The
server rolls it back to the checkpoint, rebuilds it in FP64 from that state
(mfem_gpu_scene_snapshot / restore) and the FP64 scene takes the failed
step again.  A scene that fails in FP64 leaves with its status, as the
reference would stop.  Scenes of one precision share a batch.

No counterpart in the reference, which steps one scene per process.
"""
import concurrent.futures as cf
import copy
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi, gpu


@dataclass
class Request:
    spec: object
    steps: int
    arrival: float = 0.0           # seconds after the server starts
    rid: int = -1
    footprint: int = 0
    # filled by the server
    admitted_at: float = None
    done_at: float = None
    steps_done: int = 0
    step_ms: list = field(default_factory=list)    # device time of each tick it took part in
    newton: list = field(default_factory=list)
    cg: list = field(default_factory=list)
    status: int = abi.OK
    escalated_at: int = None       # timesteps taken in mixed precision before FP64
    result: dict = None


class Server:
    """Continuous-batching loop over one GPU.

    budget_bytes  device memory the admitted scenes may hold together
    keep_state    which final state arrays to return ("x", "v", "s", "R")
    escalate      continue a mixed-precision scene in FP64 after a failed
                  line search
    steps_per_tick  timesteps a tick may take per instance (each at its own
                  pace); a failed step rolls back the instance's whole tick
    tune          let batch creation run the autotuner's timings
    lanes         independent loops (threads, batches, streams) the
                  requests are dealt out to, each with budget / lanes
    """

    def __init__(self, budget_bytes, keep_state=("x",), max_scenes=4096, escalate=True, steps_per_tick=1,
                 tune=False, lanes=1):
        self.budget = int(budget_bytes)
        self.lanes = max(1, int(lanes))
        self.steps_per_tick = max(1, int(steps_per_tick))
        self.tune = bool(tune)
        self.keep = tuple(keep_state)
        self.max_scenes = max_scenes
        self.escalate = escalate
        self.queue = []
        self.ticks = []

    def submit(self, spec, steps, arrival=0.0):
        if int(steps) < 1:
            raise ValueError("a request takes at least one timestep")
        r = Request(spec=spec, steps=int(steps), arrival=float(arrival), rid=len(self.queue))
        r.footprint = gpu.footprint(spec) + self._checkpoint_bytes(spec)
        if r.footprint > self.budget:
            raise ValueError(f"request {r.rid} needs {r.footprint} bytes, over the budget")
        self.queue.append(r)
        return r.rid

    def _checkpoint_bytes(self, spec):
        """Device bytes of the per-tick checkpoint a mixed scene keeps when
        escalation is on (positions and the BDF history of x and v at 24
        bytes a vertex each, s and the quaternions at 64 bytes a tet)."""
        if not self.escalate or getattr(spec, "precision", None) != abi.PRECISION_MIXED:
            return 0
        nv = getattr(spec, "n_vertices", 0)
        nt = getattr(spec, "n_tets", 0)
        bdf = getattr(spec, "bdf_order", 1)
        return 24 * nv * (1 + 2 * bdf) + 64 * nt

    @staticmethod
    def _in_fp64(r, sc):
        """The scene rolled back to its checkpoint and rebuilt in FP64 there."""
        sc.rollback()
        snap = sc.snapshot()
        spec = copy.copy(r.spec)
        spec.precision = abi.PRECISION_FP64
        sc64 = gpu.Scene(spec)
        sc64.restore(snap)
        return spec, sc64

    def run(self, realtime=True):
        """Serves every submitted request; returns them with their results.
        realtime: arrivals follow the wall clock (else all are due at once).
        With lanes > 1 the requests are dealt out in arrival order, each to
        the lane with the least work so far (footprint x timesteps), and
        every lane runs this loop on its share of the budget in a thread of
        its own: its batches step on their own streams, so a slow instance
        holds back only its lane's ticks."""
        set_tuning = getattr(gpu, "set_tuning", None)
        if set_tuning is not None and not self.tune:
            set_tuning(0)
        t0 = time.perf_counter()
        try:
            if self.lanes <= 1:
                self.ticks += self._run_lane(self.queue, realtime, self.budget, t0)
            else:
                L = self.lanes
                share = self.budget // L
                parts, work = [[] for _ in range(L)], [0.0] * L
                for r in sorted(self.queue, key=lambda r: (r.arrival, r.rid)):
                    if r.footprint > share:
                        raise ValueError(f"request {r.rid} needs {r.footprint} bytes, over a lane's budget")
                    k = min(range(L), key=lambda j: (work[j], j))
                    parts[k].append(r)
                    work[k] += float(r.footprint) * r.steps
                with cf.ThreadPoolExecutor(max_workers=L) as lanes:
                    futs = [lanes.submit(self._run_lane, parts[k], realtime, share, t0) for k in range(L)]
                    for f in futs:
                        self.ticks += f.result()
                self.ticks.sort(key=lambda t: t[0])
        finally:
            if set_tuning is not None and not self.tune:
                set_tuning(-1)
        return sorted(self.queue, key=lambda r: r.rid)

    def _run_lane(self, requests, realtime, budget, t0):
        """The loop over one lane's requests; returns its ticks."""
        ticks = []
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        building = {}          # rid -> future(Scene)
        active = {}            # rid -> (Request, Scene)
        groups = {}            # precision -> (Batch, member rids)
        used = 0
        pool = cf.ThreadPoolExecutor(max_workers=1)
        stepper = cf.ThreadPoolExecutor(max_workers=2)
        now = lambda: time.perf_counter() - t0

        inflight = {}          # precision -> (future of its tick, member rids)

        def close_batches():
            for b, _ in groups.values():
                b.close()
            groups.clear()

        def tick(b, members):
            k = min([self.steps_per_tick] + [active[m][0].steps - active[m][0].steps_done for m in members])
            if k > 1:
                return b.step_n(k, raise_on_error=False)
            return b.step(raise_on_error=False), None

        try:
            while pending or building or active or inflight:
                # admit what has arrived and fits
                while (pending and (not realtime or pending[0].arrival <= now())
                       and used + pending[0].footprint <= budget
                       and len(active) + len(building) < self.max_scenes):
                    r = pending.pop(0)
                    used += r.footprint
                    building[r.rid] = (r, pool.submit(gpu.Scene, r.spec))
                # scenes whose build finished join their group's next tick
                for rid in [k for k, (_, f) in building.items() if f.done() or not (active or inflight)]:
                    r, f = building.pop(rid)
                    active[rid] = (r, f.result())
                    r.admitted_at = now()
                if not active and not inflight:
                    if pending and realtime:
                        time.sleep(max(0.0, min(0.01, pending[0].arrival - now())))
                    continue
                # every idle precision group with members starts its next tick:
                # the groups tick independently, each batch on its own stream
                # (the library's calls on distinct batches are thread-safe and
                # release the interpreter lock), so an FP64 group's slow steps
                # do not hold back the mixed group and the other way round
                by_prec = {}
                for k in sorted(active):
                    by_prec.setdefault(active[k][1].spec.precision, []).append(k)
                for p in [p for p in groups if p not in by_prec and p not in inflight]:
                    groups.pop(p)[0].close()
                for p in sorted(by_prec):
                    if p in inflight:
                        continue
                    key = tuple(by_prec[p])
                    b, members = groups.get(p, (None, ()))
                    if key != members:
                        if b is not None:
                            b.close()
                        b = gpu.Batch([active[k][1] for k in key])
                        groups[p] = (b, key)
                    if self.escalate and p == abi.PRECISION_MIXED:
                        for k in key:
                            active[k][1].checkpoint()
                    inflight[p] = (stepper.submit(tick, b, key), key)
                # wait for a group's tick (or for the next arrival)
                timeout = None
                if building:
                    timeout = 0.005
                elif pending and realtime:
                    timeout = max(0.0, pending[0].arrival - now())
                done_set, _ = cf.wait([f for f, _ in inflight.values()], timeout=timeout,
                                      return_when=cf.FIRST_COMPLETED)
                for p in [p for p, (f, _) in inflight.items() if f in done_set]:
                    f, key = inflight.pop(p)
                    stats, done = f.result()
                    results = []
                    for j, (k, st) in enumerate(zip(key, stats)):
                        if done is None:
                            ms = [stats[0].device_ms]
                        else:   # the device time of each timestep the scene took in the tick
                            d = done[j][done[j] >= 0]
                            ms = list(np.diff(np.concatenate([[0.0], d])))
                        results.append((k, st, ms))
                    ticks.append((now(), len(key), stats[0].device_ms))
                    finished, escalate = [], []
                    for k, st, ms in results:
                        r, sc = active[k]
                        if (self.escalate and sc.spec.precision == abi.PRECISION_MIXED
                                and st.status in (abi.ERR_LS_FAILED, abi.ERR_NONFINITE, abi.ERR_PROCRUSTES)):
                            # undo the tick: the FP64 scene takes its steps again
                            escalate.append(k)
                            continue
                        r.steps_done += len(ms)
                        r.step_ms += ms
                        r.newton.append(st.newton_iterations)
                        r.cg.append(st.cg_iterations)
                        if st.status not in (abi.OK, abi.ERR_CG_MAXITER, abi.ERR_LS_FAILED):
                            r.status = st.status
                        # a scene whose state is no longer finite leaves with its status
                        if r.steps_done >= r.steps or st.status in (abi.ERR_NONFINITE, abi.ERR_PROCRUSTES):
                            finished.append(k)
                    if finished or escalate:
                        groups.pop(p)[0].close()      # before any of its scenes is freed
                    for k in finished:
                        r, sc = active.pop(k)
                        if r.status in (abi.ERR_NONFINITE, abi.ERR_PROCRUSTES):
                            r.result = None
                        else:
                            state = sc.get_state()
                            r.result = {name: state[name] for name in self.keep}
                        r.done_at = now()
                        sc.close()
                        used -= r.footprint
                    for k in escalate:
                        r, sc = active[k]
                        spec, sc64 = self._in_fp64(r, sc)
                        sc.close()
                        fp = gpu.footprint(spec)
                        used += fp - r.footprint
                        r.footprint, r.escalated_at = fp, r.steps_done
                        active[k] = (r, sc64)
        finally:
            cf.wait([f for f, _ in inflight.values()])   # no batch closes under a tick
            close_batches()
            for r, sc in active.values():
                sc.close()
            pool.shutdown(wait=True)
            stepper.shutdown(wait=True)
        return ticks


def shard(weights, world_size, rank):
    """Indices of the requests rank `rank` serves when world_size GPUs share a
    stream: requests are independent, so they are dealt out with no exchange,
    greedily by decreasing weight (a scene's footprint, or its tets x steps)
    to the least-loaded rank, ties to the lower index and rank."""
    load = [0.0] * world_size
    mine = []
    for i in sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i)):
        r = min(range(world_size), key=lambda k: (load[k], k))
        load[r] += float(weights[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


def summary(requests, ticks, wall_s):
    """Aggregate timesteps/s and per-timestep latency percentiles."""
    steps = sum(r.steps_done for r in requests)
    lat = np.array([ms for r in requests for ms in r.step_ms]) if steps else np.zeros(1)
    req = np.array([r.done_at - r.arrival for r in requests if r.done_at is not None])
    failed = sum(1 for r in requests if r.status in (abi.ERR_NONFINITE, abi.ERR_PROCRUSTES))
    escalated = sum(1 for r in requests if r.escalated_at is not None)
    return {"requests": len(requests), "failed_requests": failed, "escalated_to_fp64": escalated,
            "timesteps": int(steps), "wall_s": wall_s,
            "timesteps_per_s": steps / wall_s if wall_s > 0 else None,
            "step_latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "request_latency_s": {"p50": float(np.percentile(req, 50)) if len(req) else None,
                                  "p99": float(np.percentile(req, 99)) if len(req) else None},
            "ticks": len(ticks), "max_batch": max((n for _, n, _ in ticks), default=0)}
