"""Benchmark of the GB300 mixed-FEM Newton timestep.

Default workload (N=1): the plain method at scale, a 60^3 cube grid at 0.01 m,
5 tets per cube (1,080,000 tets, 226,981 vertices), stable neo-Hookean
E=1e5 Pa, nu=0.45, initial positions perturbed U(+-10% of the spacing)
(seeded), bottom face pinned, BDF1 dt=1/60, Newton to 1e-5 relative residual,
Jacobi PCG to 1e-4, FP32 element work with FP64 reductions.  Synthetic data:
there is no dataset in this workload.

One JSON line on rank 0:
  value       timesteps/s of the whole job, state resident in HBM, from the
              per-step CUDA-event times of the library's stream
  e2e         the same steps again from the same starting state, through the
              C ABI with pinned host buffers: every step uploads the pinned
              vertices' targets and reads all vertex positions back
  roofline    the dominant kernel's algorithmic bytes per launch / its average
              launch time (CUDA events around every launch, in a replay of the
              timed steps from the same state: the events slow the step, so
              `value` comes from the run without them)
  error_vs_fp64  (mixed path) max |x - x_fp64| / bbox diagonal per step
              against the all-FP64 GPU path: each step retaken in FP64 from
              the mixed state before it, and an FP64 trajectory alongside
  residual_true_pcg  |b - A dx| / |b| of one solve of the PCG form the step
              runs, beside the recursive estimate it stops on
  cpu_baseline  the FP64 oracle port on the host cores: whole timesteps from
              the GPU scene's warmed state, timed with the host clock
              (about --cpu-budget seconds, at least 3 steps)
  --impl reference  the same oracle port as the reference's CPU arm: W
              untimed steps from rest, then K whole timesteps timed.

Multi-GPU (torchrun): independent replicas, one scene per rank (the path has
no exchange step); value = N * steps / max over ranks of the timed seconds.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "timesteps/s & p50/p99 step latency, batched vs plain GPU at 1e-5 residual"
UNIT = "timesteps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c5", "tri2d"],
                    help="tri2d: the 2-D path on a hanging sheet (scenes/2D/square.json settings)")
    ap.add_argument("--sheet", type=int, default=128,
                    help="squares along x of the tri2d sheet (x/4 along y, 2 triangles each)")
    ap.add_argument("--c5-duration", type=float, default=5.0,
                    help="seconds of Poisson arrivals (lambda = 20/s) in the served stream")
    ap.add_argument("--c5-steps", type=int, default=20, help="timesteps per served request")
    ap.add_argument("--c5-lanes", type=int, default=8,
                    help="independent serving loops (each its own batches, stream and thread)")
    ap.add_argument("--c5-steps-per-tick", type=int, default=4,
                    help="timesteps a serving tick may take per instance")
    ap.add_argument("--size", type=int, default=60, help="cubes per axis for c2")
    ap.add_argument("--precision", default=None, choices=["mixed", "fp64"],
                    help="default: fp64 for c1 (the beam is stated FP64 throughout), mixed otherwise")
    ap.add_argument("--solver", default="eigen-pcg-diag",
                    choices=["eigen-pcg-diag", "gpu-pcg-block", "minres-indefinite-block"])
    ap.add_argument("--formulation", default="mixed-stretch", choices=["mixed-stretch", "stretch"],
                    help="the elastic variable: MixedStretch or the standard-FEM Stretch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched-vs-plain measurement on the 64-scene mix")
    ap.add_argument("--mix-plain-steps", type=int, default=100,
                    help="timesteps per scene of the plain (one scene at a time) 64-scene mix")
    ap.add_argument("--mix-lanes", type=int, default=4,
                    help="batches the 64-scene mix is split into for the side-by-side (lanes) form")
    ap.add_argument("--mix-steps", type=int, default=100,
                    help="timesteps per scene of the batched 64-scene mix (its stated 100)")
    ap.add_argument("--no-error", action="store_true",
                    help="skip the error-vs-FP64 replay and the true PCG residual")
    ap.add_argument("--error-steps", type=int, default=10,
                    help="steps of the error-vs-FP64 replay (at most --steps)")
    ap.add_argument("--cpu-budget", type=float, default=25.0,
                    help="seconds of whole CPU timesteps in the cpu_baseline leg (at least 3 steps)")
    ap.add_argument("--ref-budget", type=float, default=300.0,
                    help="seconds of timed steps in the reference arm before it stops early")
    ap.add_argument("--c2-reading", default="jittered-rest", choices=["jittered-rest", "perturbed-initial"],
                    help="C2's 'initial vertex positions perturbed': a jittered rest mesh starting "
                         "at rest, or a regular rest grid with perturbed (pre-strained) initial positions")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--pcg-kernel", default="auto", choices=["persistent", "split", "fused", "auto"],
                    help="auto: the batch picks fused or split by its PCG tile count")
    args = ap.parse_args()
    if args.precision is None:
        args.precision = "fp64" if args.config == "c1" else "mixed"
    return args


# ----------------------------------------------------------------- ranks --
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allsum(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------- byte models --
def kernel_bytes(kind, sizes, rsz, cg_per_launch=None):
    """Algorithmic bytes per launch (each array read or written once).
    k_cg_solve runs a whole PCG solve: cg_per_launch iterations of SpMV +
    update."""
    nt, nv, nf, nnzb, n_inc, nnz_m = (sizes[k] for k in ("nt", "nv", "nf", "nnzb", "n_inc", "nnz_m"))
    if kind == "k_cg_solve":
        if not cg_per_launch:
            return None
        return cg_per_launch * (kernel_bytes("k_cg_spmv", sizes, rsz) + kernel_bytes("k_cg_update", sizes, rsz))
    if kind == "k_cg_spmv":
        # values + block cols + row ptr, z and p_prev read, Ap and p written
        return nnzb * (9 * rsz + 4) + 4 * (nf + 1) + 4 * 3 * nf * rsz
    if kind == "k_cgf_iter":
        # one pass of the matrix; own rows (Jacobi, scaled form): r, w, s, p,
        # x and the preconditioner read, r, w, s, p, x written (neighbour
        # values come from caches)
        return nnzb * (9 * rsz + 4) + 4 * (nf + 1) + 11 * 3 * nf * rsz
    if kind == "k_cg_update":
        # x (rw), r (rw), p, Ap, z (w), Jacobi diagonal
        return 8 * 3 * nf * rsz
    if kind == "k_elem_update":
        # tets, dphi, vol/mu/lam, s, rotation (rw), S (w), element record (w), x
        return nt * (16 + 9 * rsz + 3 * rsz + 6 * rsz + 8 * rsz + 6 * rsz + 92 * rsz) + 24 * nv
    if kind == "k_assemble":
        return (nt * 92 * rsz + nnzb * (9 * rsz + rsz + 4) + 8 * n_inc + 4 * (nf + 1) * 2 +
                nnz_m * 12 + 48 * nv + 3 * nf * rsz + 3 * nf * rsz)
    if kind == "k_local_solve":
        return nt * (16 + 9 * rsz + 3 * rsz + 4 * rsz + 6 * rsz * 4) + 3 * nf * rsz + nnz_m * 12 + 48 * nv
    if kind == "k_ls_energy":
        return nt * (16 + 9 * rsz + 3 * rsz + 4 * rsz + 6 * rsz * 3) + 3 * nf * rsz + nnz_m * 12 + 48 * nv
    if kind == "k_elem_fem":
        # tets, dphi, vol/mu/lam, x; element record (w)
        return nt * (16 + 9 * rsz + 3 * rsz + 92 * rsz) + 24 * nv
    if kind == "k_mr_elem":
        # ds/dx (72) and H (21) in Real, vol, tets, free_map; FP64: wn (12 own
        # + 12 gathered x), v (rw), vn (rw), w (w), the pending p / x update
        # (w, p1, p2 read, p0 written, x rw: 72), shares y (12 w)
        return nt * (94 * rsz + 32 + 8 * (24 + 24 + 24 + 12 + 72 + 12))
    if kind == "k_mr_vert":
        # mass row (col, value, neighbour wn), incidences and their shares;
        # own x rows: v, vn (rw), wn (r), w (w), the pending update (6 x 3)
        return nnz_m * (4 + rsz + 24) + n_inc * (8 + 24) + nf * 8 * 3 * (2 + 2 + 1 + 1 + 6)
    if kind == "k_mr_update":
        # vn (rw), v (r), wn (w) for 12 element and 3 row entries; (vol H)^-1
        # and S_ee^-1 (42 doubles), 1/m per row
        return nt * 8 * (12 * 4 + 42) + nf * 8 * (3 * 4 + 1)
    return None


def read_traffic(kernel, workload, cg_per_launch=None):
    """DRAM bytes per launch from the committed ncu summary, if present.
    For the whole-PCG kernel the summary holds bytes per PCG iteration,
    scaled here by this run's PCG iterations per launch."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        key, _, val = ln.strip().partition(":")
        try:
            if key == "dram_bytes_per_launch":
                return float(val.split()[0])
            if key == "dram_bytes_per_pcg_iteration" and cg_per_launch:
                return float(val.split()[0]) * cg_per_launch
        except (ValueError, IndexError):
            return None
    return None


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------- workloads --
def make_spec(args, precision):
    from mfem_gb300 import abi, configs
    prec = abi.PRECISION_MIXED if precision == "mixed" else abi.PRECISION_FP64
    solver = {"eigen-pcg-diag": abi.SOLVER_EIGEN_CG_DIAG, "gpu-pcg-block": abi.SOLVER_GPU_PCG_BLOCK,
              "minres-indefinite-block": abi.SOLVER_MINRES_ID}[args.solver]
    kern = {"persistent": abi.PCG_KERNEL_PERSISTENT, "split": abi.PCG_KERNEL_SPLIT,
            "fused": abi.PCG_KERNEL_FUSED, "auto": abi.PCG_KERNEL_AUTO}[args.pcg_kernel]
    form = abi.FORMULATION_STRETCH if args.formulation == "stretch" else abi.FORMULATION_MIXED_STRETCH
    kw = dict(precision=prec, linear_solver=solver, pcg_kernel=kern, formulation=form)
    tag = ("_minres" if args.solver == "minres-indefinite-block" else "") + \
          ("_stretch" if args.formulation == "stretch" else "")
    if args.config == "c1":
        return configs.beam_c1(**kw), "beam_c1_200tets" + tag
    if args.config == "c3":
        return configs.stress_c3(**kw), "stress_c3_135k" + tag
    n = args.size
    literal = args.c2_reading == "perturbed-initial"
    reading = "_perturbed_initial" if literal else "_jittered_rest"
    return (configs.cube_c2(n=n, perturb_initial_only=literal, **kw),
            f"cube_c2_{n}^3_{5 * n ** 3}tets{reading}" + tag)


def scene_sizes(spec, scene):
    V, T = spec.V_rest, spec.tets
    nv = V.shape[0]
    fixed = spec.is_fixed if spec.is_fixed is not None else np.zeros(nv, np.int32)
    # vertex adjacency nnz (mass CSR) and incidences of free rows
    deg = np.zeros(nv, np.int64)
    np.add.at(deg, T.ravel(), 1)
    n_inc = int(deg[fixed == 0].sum())
    T64 = T.astype(np.int64)
    pairs = (T64[:, :, None] * nv + T64[:, None, :]).ravel()
    nnz_m = int(np.unique(pairs).size)
    return dict(nt=T.shape[0], nv=nv, nf=scene.n_free, nnzb=scene.nnzb, n_inc=n_inc, nnz_m=nnz_m)


# ------------------------------------------------------------ CPU steps --
def cpu_steps(spec, threads, budget_s, min_steps, max_steps, warmup=0, state=None):
    """Whole timesteps of the FP64 oracle on the host cores, each timed with
    the host clock: `warmup` untimed steps, then timed steps until max_steps
    have run or budget_s has passed (at least min_steps).  From `state` (x,
    v, s, R of a scene, e.g. the GPU scene's warmed state) when given, else
    from the workload's initial state."""
    import oracle
    threads = oracle.set_threads(threads)
    t_make = time.perf_counter()
    sc = oracle.OracleScene(spec)
    if state is not None:
        sc.set_state(x=state["x"], v=state["v"], s=state["s"], R=state["R"])
    make_s = time.perf_counter() - t_make
    for _ in range(warmup):
        sc.step()
    secs, newton, cg = [], [], []
    t0 = time.perf_counter()
    while len(secs) < max_steps and (len(secs) < min_steps or time.perf_counter() - t0 < budget_s):
        t = time.perf_counter()
        st = sc.step()
        secs.append(time.perf_counter() - t)
        newton.append(int(st.newton_iterations))
        cg.append(int(st.cg_iterations))
    return {"threads": threads, "steps": len(secs), "seconds": float(sum(secs)), "step_s": secs,
            "newton_iterations": newton, "cg_iterations": cg, "warmup": warmup,
            "scene_build_s": make_s, "n_free": sc.n_free, "nnzb": sc.nnzb}


def cpu_line(res, workload, start):
    value = res["steps"] / res["seconds"]
    return {"value": value, "unit": UNIT, "cores": res["threads"], "kind": "port",
            "steps_timed": res["steps"],
            "sample": (f"FP64 oracle (the project's C++/OpenMP restatement of the reference step) on "
                       f"{res['threads']} host threads, {workload}: {res['steps']} whole timesteps from "
                       f"{start}, {res['seconds']:.1f} s in all ({res['seconds'] / res['steps']:.2f} s a "
                       f"step; {np.mean(res['newton_iterations']):.2f} Newton and "
                       f"{np.mean(res['cg_iterations']):.0f} PCG iterations a step)"),
            "newton_iterations": res["newton_iterations"], "cg_iterations": res["cg_iterations"],
            "step_s": [round(t, 3) for t in res["step_s"]]}


def workload_config(args, spec, workload, nf, nnzb, ws):
    """The `config` object of both arms (the same workload, whatever the arm
    computes in)."""
    big = args.config == "c2" and args.size >= 40
    return {"workload": workload, "tets": int(spec.n_tets), "vertices": int(spec.n_vertices),
            "free_dofs": 3 * int(nf), "blocks": int(nnzb), "solver": args.solver,
            "formulation": args.formulation,
            "newton_residual_tolerance": spec.newton_residual_tolerance,
            "pcg_tolerance": spec.iterative_solver_tolerance,
            "l2": ("working set > L2 (about 1 GB per step); no flush" if big else
                   "working set within L2; no flush"),
            "parallelism": f"replicas{ws}"}


def run_reference(args):
    """The reference arm: the FP64 oracle port (the reference itself does not
    build here) stepping the same workload on all host cores, W untimed
    warm-up steps from the initial state, then K whole timesteps timed."""
    ws, rank, _, pg = dist_setup()
    if rank != 0:
        return 0
    import oracle  # noqa: F401  (the reference arm is the FP64 port on the host cores)
    threads = args.cpu_threads or os.cpu_count()
    spec, workload = make_spec(args, "fp64")
    res = cpu_steps(spec, threads, budget_s=args.ref_budget, min_steps=min(args.steps, 3),
                    max_steps=args.steps, warmup=args.warmup)
    cb = cpu_line(res, workload, f"the state after {args.warmup} untimed steps from rest")
    value = cb["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": res["steps"], "steps_requested": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, spec, workload, res["n_free"], res["nnzb"], ws),
        "precision": "fp64",
        "p50_ms": 1000.0 * float(np.percentile(res["step_s"], 50)),
        "p99_ms": 1000.0 * float(np.percentile(res["step_s"], 99)),
        "newton_iterations_per_step": float(np.mean(res["newton_iterations"])),
        "cg_iterations_per_step": float(np.mean(res["cg_iterations"])),
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def error_vs_fp64(args, spec_fp64, scene, state0, steps):
    """Error of the mixed path against the all-FP64 GPU path, outside the
    timed region.  same_state: each step taken in FP64 from the mixed
    path's state before it; trajectory: an FP64 scene stepped from the same
    starting state alongside.  Both as max |x - x_fp64| over the bounding-box
    diagonal of x_fp64, per step."""
    from mfem_gb300 import gpu
    f64 = gpu.Scene(spec_fp64)
    traj = gpu.Scene(spec_fp64)
    scene.set_state(x=state0["x"], v=state0["v"], s=state0["s"], R=state0["R"])
    traj.set_state(x=state0["x"], v=state0["v"], s=state0["s"], R=state0["R"])
    same, along, t64 = [], [], []
    for _ in range(steps):
        before = scene.get_state()
        scene.step()
        xm = scene.positions()
        f64.set_state(x=before["x"], v=before["v"], s=before["s"], R=before["R"])
        t = time.perf_counter()
        f64.step()
        t64.append(time.perf_counter() - t)
        x64 = f64.positions()
        diag = float(np.linalg.norm(np.ptp(x64, axis=0)))
        same.append(float(np.abs(xm - x64).max()) / diag)
        traj.step()
        xt = traj.positions()
        along.append(float(np.abs(xm - xt).max()) / float(np.linalg.norm(np.ptp(xt, axis=0))))
    f64.close()
    traj.close()
    return {"metric": "max |x - x_fp64| / bbox diagonal", "steps": steps,
            "same_state_max": max(same), "same_state": same,
            "trajectory_max": max(along), "trajectory": along,
            "fp64_gpu_step_s": float(np.mean(t64)),
            "note": "same_state: one FP64 GPU step from the mixed state before each step; "
                    "trajectory: FP64 GPU scene stepped from the same starting state"}


def true_pcg_residual(scene):
    """The true residual |b - A dx| / |b| of one solve of the scene's PCG form
    on the system assembled at the scene's current state (A as the device
    holds it), beside the recursive estimate the solver stops on."""
    rp, col, val, rhs = scene.get_system()
    dx, it, rec = scene.pcg(rhs)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    y = np.zeros((n, 3))
    np.add.at(y, rows, np.einsum("kij,kj->ki", val, dx.reshape(-1, 3)[col]))
    true = float(np.linalg.norm(rhs - y.ravel()) / np.linalg.norm(rhs))
    return {"true": true, "recursive": float(rec), "iterations": int(it),
            "tolerance": float(scene.spec.iterative_solver_tolerance)}


# ----------------------------------------------------------------- ours --
def run_ours(args):
    ws, rank, local, pg = dist_setup()
    from mfem_gb300 import abi, gpu
    from mfem_gb300.build import build
    if rank == 0:
        build()
    barrier(pg)
    import ctypes
    from mfem_gb300._lib import load
    L = load()
    if ws > 1:
        from mfem_gb300._lib import check
        check(L.mfem_gpu_set_device(local), "set_device")
    spec, workload = make_spec(args, args.precision)
    scene = gpu.Scene(spec)
    batch_h = scene.solo_batch_handle()
    sizes = scene_sizes(spec, scene)
    rsz = 4 if args.precision == "mixed" else 8

    for _ in range(args.warmup):
        st = scene.step()
    state0 = scene.get_state()
    barrier(pg)
    sampler = ClockSampler(local)
    sampler.start()
    ms, stats = [], []
    k_before = gpu.kernel_stats(batch_h)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = scene.step()
        ms.append(st.device_ms)
        stats.append(st.as_dict())
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    k_after = gpu.kernel_stats(batch_h)
    # the library's launches in the timed region, by kernel (counted on the
    # host; the device-driven PCG loop's launches as its bodies report them)
    timed_launches = {k: int(k_after[k][1] - k_before[k][1]) for k in k_after if k_after[k][1] > k_before[k][1]}
    dev_s = sum(ms) / 1000.0
    dev_s_max = allmax(pg, dev_s)
    value = ws * args.steps / dev_s_max

    # ---- end to end through the C ABI with host buffers: the same steps
    # again from the state the timed region started from
    e2e = None
    if not args.no_e2e:
        import torch
        pins = scene.pinned()
        scene.set_state(x=state0["x"], v=state0["v"], s=state0["s"], R=state0["R"])
        pin_host = torch.from_numpy(np.ascontiguousarray(state0["x"][pins])).pin_memory()
        x_host = torch.zeros((scene.n_vertices, 3), dtype=torch.float64).pin_memory()
        dptr = ctypes.POINTER(ctypes.c_double)
        e2e_stats = []
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            L.mfem_gpu_scene_set_pins(scene.handle, ctypes.cast(pin_host.data_ptr(), dptr))  # H2D
            e2e_stats.append(scene.step())
            L.mfem_gpu_scene_get_state(scene.handle, ctypes.cast(x_host.data_ptr(), dptr),
                                       None, None, None, None)                          # D2H
        e2e_s = allmax(pg, time.perf_counter() - t0)
        e2e = {"value": ws * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(pin_host.numel() * 8),
               "d2h_bytes_per_step": int(x_host.numel() * 8), "steps": args.steps,
               "newton_iterations_per_step": float(np.mean([t.newton_iterations for t in e2e_stats])),
               "cg_iterations_per_step": float(np.mean([t.cg_iterations for t in e2e_stats])),
               "host_buffers": "pinned (cudaHostAlloc through torch.pin_memory)"}
        if spec.bc_type not in (abi.BC_NULL, abi.BC_HANG, abi.BC_HANGENDS) and len(pins):
            e2e["note"] = ("the caller drives the pins: each step uploads their starting positions, which "
                           "replaces the scripted boundary motion the timed value follows, so the two "
                           "figures step different problems")

    # ---- per-kernel CUDA events: a replay of the same steps from the same
    # state with an event pair around every launch (the events slow the
    # step, so the timed region above runs without them)
    scene.set_state(x=state0["x"], v=state0["v"], s=state0["s"], R=state0["R"])
    gpu.set_profiling(batch_h, True)
    prof_ms = []
    for _ in range(args.steps):
        prof_ms.append(scene.step().device_ms)
    kstats = gpu.kernel_stats(batch_h)
    gpu.set_profiling(batch_h, False)
    prof_s = sum(prof_ms) / 1000.0

    # ---- roofline of the dominant kernel
    cg_total = float(sum(s["cg_iterations"] for s in stats))
    cg_per_solve = cg_total / kstats["k_cg_solve"][1] if kstats.get("k_cg_solve", (0, 0))[1] else None
    dom = max(kstats, key=lambda k: kstats[k][0])
    dom_ms, dom_n = kstats[dom]
    abytes = kernel_bytes(dom, sizes, rsz, cg_per_solve)
    peak, peak_src = measured_peak()
    achieved = abytes / (dom_ms / dom_n / 1e3) / 1e9 if abytes and dom_n else None
    if dom == "k_cg_solve" and cg_per_solve:
        # per PCG iteration, so that the figure compares with the split kernels
        roof_note = f"k_cg_solve: {cg_per_solve:.1f} PCG iterations per launch"
    else:
        roof_note = None
    roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "note": roof_note,
            "frac": achieved / peak if achieved else None,
            "traffic": read_traffic(dom, "c2", cg_per_solve) if args.config == "c2" and args.size == 60 else None,
            "algorithmic_bytes_per_launch": abytes, "avg_launch_us": 1e3 * dom_ms / dom_n,
            "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"}
    per_kernel = {}
    for k, (kms, kn) in kstats.items():
        if kn:
            b = kernel_bytes(k, sizes, rsz, cg_per_solve)
            per_kernel[k] = {"ms": round(kms, 3), "launches": kn,
                             "share": round(kms / max(prof_s * 1e3, 1e-9), 4),
                             "GBps": round(b / (kms / kn / 1e3) / 1e9, 1) if (b and kms > 0) else None}
    launches = int(sum(timed_launches.values()))

    newton = float(np.mean([s["newton_iterations"] for s in stats]))
    cgits = float(np.mean([s["cg_iterations"] for s in stats]))
    pcg_shape = dict(zip(("stages", "keep", "unroll", "pdl"), gpu.get_pcg_shape(batch_h)))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        # mixed: FP32 element work, matrix and SpMV; positions, s, the residual
        # chain and every reduction in float-float (df64, ~48-bit significand,
        # FP32 exponent range)
        "dtype": "f32+df64" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": workload_config(args, spec, workload, sizes["nf"], sizes["nnzb"], ws),
        "precision": args.precision, "pcg_kernel": args.pcg_kernel,
        "pcg_kernel_resolved": ("fused" if kstats.get("k_cgf_iter", (0, 0))[1] else
                                "split" if kstats.get("k_cg_spmv", (0, 0))[1] else
                                "persistent" if kstats.get("k_cg_solve", (0, 0))[1] else None),
        "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
        "wall_ms_per_step": 1000.0 * wall / args.steps,
        "newton_iterations_per_step": newton, "cg_iterations_per_step": cgits,
        "residual_rel_last": stats[-1]["residual"] / max(stats[-1]["residual0"], 1e-300),
        # the last linear solve of each timed step against its tolerance (a
        # solver that stops on its iteration limit shows here)
        "linear_solve_rel_residual": [float(st["cg_error"]) for st in stats],
        "linear_solve_converged_steps": int(sum(1 for st in stats
                                                if st["cg_error"] <= spec.iterative_solver_tolerance)),
        "clocks": clocks, "e2e": e2e, "roofline": roof, "gpu_launches": launches,
        "gpu_launches_by_kernel": timed_launches,
        "profiled_replay_ms_per_step": 1000.0 * prof_s / args.steps,
        "kernels": per_kernel,
        "pcg_shape": pcg_shape,
        "autotune": gpu.tune_report(batch_h),
    }
    # ---- error against the all-FP64 GPU path and the true PCG residual
    # (outside the timed region)
    if args.precision == "mixed" and not args.no_error and args.formulation == "mixed-stretch" \
            and args.solver != "minres-indefinite-block":
        spec64, _ = make_spec(args, "fp64")
        line["error_vs_fp64"] = error_vs_fp64(args, spec64, scene, state0,
                                              min(args.steps, args.error_steps))
    if not args.no_error and args.solver != "minres-indefinite-block":
        line["residual_true_pcg"] = true_pcg_residual(scene)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # whole FP64 oracle timesteps from the GPU scene's warmed state (the
        # state the timed region started from)
        threads = args.cpu_threads or os.cpu_count()
        ref_spec, _ = make_spec(args, "fp64")
        res = cpu_steps(ref_spec, threads, budget_s=args.cpu_budget, min_steps=min(3, args.steps),
                        max_steps=args.steps, state=state0)
        line["cpu_baseline"] = cpu_line(res, workload, f"the GPU scene's state after {args.warmup} steps")
    scene.close()
    if rank == 0 and ws == 1 and not args.no_batch and args.config == "c2":
        from mfem_gb300 import configs
        line["batch_mix"] = run_batch_mix(args, gpu, abi, configs)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_batch_mix(args, gpu, abi, configs):
    """The 64-scene mix (cube grids 4..30 per axis, random materials and
    pinned face, seeded).  After the same 2 warm-up steps:

    batched    the stated 100 timesteps of every scene in one
               mfem_gpu_batch_step_n call, each scene at its own pace
    batched_3  the same form over 3 timesteps from the same state, beside
    lockstep   the one-step batch form (every scene waits for the slowest
               scene's Newton loop each step), 3 steps from that state, and
    plain      each scene alone through mfem_gpu_scene_step, one after the
               other, over the same timesteps as `batched` (--mix-plain-steps;
               its first 3 steps are also reported beside batched_3)
    timesteps/s counts scene-steps; device time from CUDA events.  Latency:
    the device time between a scene's consecutive steps in the 100-step
    call.  A scene whose step ends non-finite is retired (its remaining
    steps are not taken and not counted)."""
    kern = {"persistent": abi.PCG_KERNEL_PERSISTENT, "split": abi.PCG_KERNEL_SPLIT,
            "fused": abi.PCG_KERNEL_FUSED, "auto": abi.PCG_KERNEL_AUTO}[args.pcg_kernel]
    specs = configs.batch_c4(pcg_kernel=kern)
    n = len(specs)
    tets = int(sum(s.n_tets for s in specs))
    warm, steps, short = 2, args.mix_steps, 3
    scenes = [gpu.Scene(s) for s in specs]
    batch = gpu.Batch(scenes)
    for _ in range(warm):
        batch.step(raise_on_error=False)
    snap = [s.snapshot() for s in scenes]

    def restore():
        for sc, sn in zip(scenes, snap):
            sc.restore(sn)

    st3, d3 = batch.step_n(short, raise_on_error=False)
    b3 = int((d3 >= 0).sum()) / (st3[0].device_ms / 1e3)
    restore()
    ls_ms = [batch.step(raise_on_error=False)[0].device_ms for _ in range(short)]
    lockstep = n / (float(np.mean(ls_ms)) / 1e3)
    restore()
    stats, done = batch.step_n(steps, raise_on_error=False)
    batched_ms = stats[0].device_ms
    batch.close()
    # the same 100 timesteps from the same state with the scenes in lanes:
    # balanced batches stepped side by side on their own streams
    restore()
    lanes = gpu.Lanes(scenes, lanes=args.mix_lanes)
    t_l = time.perf_counter()
    lstats, ldone = lanes.step_n(steps, raise_on_error=False)
    lanes_s = time.perf_counter() - t_l
    lanes_ms = max(st.device_ms for st in lstats)
    lanes.close()
    lanes_steps = int((ldone >= 0).sum())
    for s in scenes:
        s.close()
    taken = done >= 0
    lat = np.diff(np.concatenate([np.zeros((n, 1)), np.where(taken, done, np.nan)], axis=1), axis=1)
    lat = lat[np.isfinite(lat)]
    scene_steps = int(taken.sum())
    newton = float(np.sum([st.newton_iterations for st in stats])) / max(scene_steps, 1)
    failed = [i for i, st in enumerate(stats) if st.status not in (abi.OK, abi.ERR_LS_FAILED, abi.ERR_CG_MAXITER)]
    finish = np.array([float(d[t].max()) if t.any() else 0.0 for d, t in zip(done, taken)])
    slowest = list(np.argsort(-finish)[:3])
    batched = scene_steps / (batched_ms / 1e3)
    plain_ms, plain_n, plain_steps = 0.0, 0, args.mix_plain_steps
    p3_ms, p3_n = 0.0, 0
    scene_ms = []
    for sp in specs:
        s = gpu.Scene(sp)
        retired = False
        for _ in range(warm):
            if s.step(raise_on_error=False).status in (abi.ERR_NONFINITE, abi.ERR_PROCRUSTES):
                retired = True
                break
        own = 0.0
        for k in range(0 if retired else plain_steps):
            st = s.step(raise_on_error=False)
            plain_ms += st.device_ms
            own += st.device_ms
            plain_n += 1
            if k < short:
                p3_ms += st.device_ms
                p3_n += 1
            if st.status in (abi.ERR_NONFINITE, abi.ERR_PROCRUSTES):
                break  # retired, as in the batched form
        scene_ms.append(own)
        s.close()
    plain = plain_n / (plain_ms / 1e3)
    plain_3 = p3_n / (p3_ms / 1e3)
    # a batch finishes no sooner than its slowest scene's chain of Newton and
    # PCG iterations, and with every scene at its own pace alone the
    # batched/plain ratio cannot pass (sum of the scenes' plain times) /
    # (the slowest scene's plain time)
    return {"workload": f"batch_c4_{n}_scenes", "scenes": n, "tets_total": tets,
            "batched": {"value": batched, "unit": UNIT, "steps": steps, "warmup": warm,
                        "form": "mfem_gpu_batch_step_n (each scene at its own pace)",
                        "ms_total": batched_ms, "scene_steps": scene_steps,
                        "newton_per_scene_step": newton,
                        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                        "scenes_done_ms_p50_p90_max": [float(np.percentile(finish, 50)),
                                                       float(np.percentile(finish, 90)), float(finish.max())],
                        "failed_scenes": [{"scene": int(i), "tets": specs[i].n_tets, "status": int(stats[i].status),
                                           "steps_done": int(taken[i].sum())} for i in failed],
                        "slowest_scenes": [{"scene": int(i), "tets": specs[i].n_tets, "done_ms": float(finish[i]),
                                            "newton": int(stats[i].newton_iterations),
                                            "cg": int(stats[i].cg_iterations)} for i in slowest]},
            "batched_lanes": {"value": lanes_steps / (lanes_ms / 1e3), "unit": UNIT, "steps": steps,
                              "lanes": len(lanes.parts), "scene_steps": lanes_steps,
                              "ms_total": lanes_ms, "wall_s": lanes_s,
                              "form": "mfem_gpu_batches_step_n: tets-balanced batches side by side, each on its "
                                      "own stream (the lane of the smallest scenes at the highest priority)"},
            "batched_3": {"value": b3, "unit": UNIT, "steps": short},
            "lockstep": {"value": lockstep, "unit": UNIT, "steps": short,
                         "ms_per_batch_step": float(np.mean(ls_ms))},
            "plain": {"value": plain, "unit": UNIT, "steps_per_scene": plain_steps, "warmup": warm,
                      "scene_steps": plain_n, "ms_per_scene_step": plain_ms / max(plain_n, 1),
                      "slowest_scene_ms": float(max(scene_ms)), "slowest_scene": int(np.argmax(scene_ms)),
                      "ratio_bound_sum_over_slowest": float(sum(scene_ms) / max(max(scene_ms), 1e-9))},
            "plain_3": {"value": plain_3, "unit": UNIT, "steps_per_scene": short, "scene_steps": p3_n},
            "batched_vs_plain": batched / plain,
            "batched_lanes_vs_plain": (lanes_steps / (lanes_ms / 1e3)) / plain,
            "batched_3_vs_plain_3": b3 / plain_3,
            "lockstep_vs_plain_3": lockstep / plain_3}


def run_served(args):
    """The served stream (C5 shape, scaled in time): Poisson arrivals at 20/s,
    cube-grid scenes of 1e3..5e5 tets (log-uniform), random materials and one
    pinned face, admitted against a 150 GB budget and stepped by continuous
    batching.  Aggregate timesteps/s, per-timestep and per-request latency;
    beside it the same requests' first timesteps stepped one scene at a time."""
    ws, rank, _, pg = dist_setup()
    from mfem_gb300 import abi, configs, gpu, server
    from mfem_gb300.build import build
    if rank == 0:
        build()
    barrier(pg)
    kern = {"persistent": abi.PCG_KERNEL_PERSISTENT, "split": abi.PCG_KERNEL_SPLIT,
            "fused": abi.PCG_KERNEL_FUSED, "auto": abi.PCG_KERNEL_AUTO}[args.pcg_kernel]
    stream = configs.stream_c5(duration=args.c5_duration, steps=args.c5_steps)
    for _, sp, _ in stream:
        sp.pcg_kernel = kern
    # N GPUs: the requests are dealt out by work (tets x timesteps), no exchange
    mine = server.shard([sp.n_tets * n for _, sp, n in stream], ws, rank)
    srv = server.Server(budget_bytes=150e9, lanes=args.c5_lanes, steps_per_tick=args.c5_steps_per_tick)
    for i in mine:
        t, sp, n = stream[i]
        srv.submit(sp, n, arrival=t)
    barrier(pg)
    t0 = time.perf_counter()
    out = srv.run(realtime=True)
    wall = allmax(pg, time.perf_counter() - t0)
    summ = server.summary(out, srv.ticks, wall)
    if ws > 1:
        total = allsum(pg, summ["timesteps"])
        summ = dict(summ, timesteps_all_ranks=int(total), timesteps_per_s=total / wall,
                    requests_all_ranks=int(allsum(pg, summ["requests"])))
    # plain: the first requests served one scene at a time (the same loop
    # with one scene per tick, all their timesteps), by device time
    sample = out[: min(len(out), 16)]
    plain_srv = server.Server(budget_bytes=150e9, max_scenes=1)
    for r in sample:
        plain_srv.submit(r.spec, r.steps)
    t1 = time.perf_counter()
    plain_out = plain_srv.run(realtime=False)
    plain_wall = time.perf_counter() - t1
    plain_ms = sum(ms for r in plain_out for ms in r.step_ms)
    plain_n = sum(r.steps_done for r in plain_out)
    plain = plain_n / (plain_ms / 1e3)
    # the served stream's own device time (the sum of its ticks)
    served_dev_s = sum(ms for _, _, ms in srv.ticks) / 1e3
    line = {"metric": METRIC, "value": summ["timesteps_per_s"], "unit": UNIT, "n_gpus": ws,
            "steps": args.c5_steps, "warmup": 0, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32+df64" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": f"served_stream_c5_{args.c5_duration:g}s_{args.c5_steps}steps",
                       "arrival_rate_per_s": 20.0, "tets_range": [1e3, 5e5],
                       "budget_bytes": 150e9, "pcg_kernel": args.pcg_kernel,
                       "lanes": args.c5_lanes, "steps_per_tick": args.c5_steps_per_tick},
            "served": summ,
            "plain": {"value": plain, "unit": UNIT, "wall_value": plain_n / plain_wall,
                      "sample": f"all timesteps of the first {len(sample)} requests, one scene at a time "
                                "(value by device time, wall_value by the host clock)"},
            "served_device_timesteps_per_s": summ["timesteps"] / served_dev_s if served_dev_s > 0 else None,
            "served_vs_plain": summ["timesteps_per_s"] / plain if plain else None,
            "tets_total": int(sum(r.spec.n_tets for r in out))}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ 2-D --
def tri2d_workload(nx):
    """A hanging sheet with the settings of the reference's 2-D scene
    (scenes/2D/square.json: dt 0.0333, hangends ratio 0.01 on x, SNH
    E = 1e5 Pa, nu = 0.45, rho = 1e3, cholmod, i.e. the Jacobi PCG at 1e-10,
    30 Newton and 20 line-search iterations): nx x nx/4 squares of side 1/nx."""
    from mfem_gb300 import abi
    from mfem_gb300.desc import Tri2dSpec
    from mfem_gb300.meshgen import enu_to_lame, square_grid
    ny = max(nx // 4, 1)
    V, T = square_grid(nx, ny, 1.0 / nx)
    lam, mu = enu_to_lame(1e5, 0.45)
    spec = Tri2dSpec(V_rest=V, tris=T, mu=np.full(len(T), float(mu)), lam=np.full(len(T), float(lam)),
                     density_const=1000.0, bc_type=abi.BC_HANGENDS, bc_ratio=0.01, bc_axis=0,
                     dt=0.0333, body_force=(0.0, float(np.float32(-9.8))), max_newton_iterations=30,
                     max_linesearch_iterations=20, max_iterative_solver_iters=10000,
                     iterative_solver_tolerance=1e-10)
    return spec, f"sheet2d_{nx}x{ny}_{len(T)}tris"


def tri2d_kernel_bytes(name, spec, n_free, nnzb, cg_per_launch):
    """Algorithmic bytes per launch of the 2-D kernels (FP64, each array read
    or written once; positions gathered once per vertex)."""
    nt, nv, nf = spec.n_tris, spec.n_vertices, n_free
    if name == "t2_elem":      # corners, dphi/dX, vol/mu/lambda/material, s, positions; 94 doubles out
        return nt * (12 + 48 + 28 + 24) + nv * 20 + nt * 94 * 8
    if name == "t2_pcg":       # per iteration: BCSR values + columns + row pointers, ~28 vector passes
        return (cg_per_launch or 0) * (36 * nnzb + 4 * nf + 224 * nf) + 64 * nf
    if name == "t2_local":
        return nt * (12 + 48 + 8 + 96 + 72 + 72 + 24 + 24 + 48) + nf * 16
    if name == "t2_energy":
        return nt * (12 + 48 + 8 + 16 + 24 + 24 + 24 + 8) + nv * 68 + nt * 16
    if name == "t2_rows":
        return 9 * nt * 36 + nnzb * 44 + nf * 48 + nv * 16
    return None


def run_tri2d(args):
    """The 2-D path's bench line: the same contract as the 3-D line on the
    tri2d sheet (FP64; replicas for N > 1)."""
    import ctypes
    ws, rank, local, pg = dist_setup()
    from mfem_gb300.build import build
    if rank == 0:
        build()
    barrier(pg)
    from mfem_gb300 import abi
    from mfem_gb300._lib import check, load
    from mfem_gb300.tri2d import Tri2dScene
    L = load()
    if ws > 1:
        check(L.mfem_gpu_set_device(local), "set_device")
    spec, workload = tri2d_workload(args.sheet)

    # timed: resident state, CUDA-event time of every step
    sc = Tri2dScene(spec)
    for _ in range(args.warmup):
        sc.step()
    before = sc.kernel_stats()
    barrier(pg)
    sampler = ClockSampler(local)
    sampler.start()
    ms, stats = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = sc.step()
        ms.append(st.device_ms)
        stats.append(st.as_dict())
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    after = sc.kernel_stats()
    launches = int(sum(after[k][1] - before[k][1] for k in after))
    dev_s_max = allmax(pg, sum(ms) / 1000.0)
    value = ws * args.steps / dev_s_max

    # end to end: the same steps on a fresh scene through the C ABI, each
    # step's positions read into a pinned host buffer
    e2e = None
    if not args.no_e2e:
        import torch
        s2 = Tri2dScene(spec)
        for _ in range(args.warmup):
            s2.step()
        x_host = torch.zeros((spec.n_vertices, 2), dtype=torch.float64).pin_memory()
        xp = ctypes.cast(x_host.data_ptr(), ctypes.POINTER(ctypes.c_double))
        st2 = abi.StepStats()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            L.mfem_gpu_tri2d_step(s2._h, ctypes.byref(st2))
            L.mfem_gpu_tri2d_get_state(s2._h, xp, None, None, None, None)
        e2e_s = allmax(pg, time.perf_counter() - t0)
        e2e = {"value": ws * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 16 * spec.n_vertices,
               "d2h_bytes_per_step": int(x_host.numel() * 8),
               "note": "h2d: the pinned vertices' positions the step uploads (the whole 2 x n "
                       "vector); d2h: all positions, read by the caller after each step"}
        s2.close()

    # per-kernel CUDA events in a replay on a fresh scene
    s3 = Tri2dScene(spec)
    for _ in range(args.warmup):
        s3.step()
    pre = s3.kernel_stats()
    s3.set_profiling(True)
    prof_ms, prof_stats = [], []
    for _ in range(args.steps):
        st3 = s3.step()
        prof_ms.append(st3.device_ms)
        prof_stats.append(st3)
    kst = s3.kernel_stats()
    s3.close()
    n_rep = {k: kst[k][1] - pre[k][1] for k in kst}   # launches of the replay
    cg_total = float(sum(t.cg_iterations for t in prof_stats))
    cg_per_launch = cg_total / max(n_rep.get("t2_pcg", 0), 1)
    timed = {k: v for k, v in kst.items() if v[0] > 0}
    dom = max(timed, key=lambda k: timed[k][0]) if timed else None
    peak, peak_src = measured_peak()
    roof = None
    per_kernel = {}
    if dom:
        for k, (kms, _) in timed.items():
            per_kernel[k] = {"ms": round(kms, 3), "launches": int(n_rep[k]),
                             "share": round(kms / max(sum(prof_ms), 1e-9), 4)}
        dom_ms = timed[dom][0]
        dom_n = max(int(n_rep[dom]), 1)
        abytes = tri2d_kernel_bytes(dom, spec, sc.n_free, sc.nnzb, cg_per_launch)
        achieved = abytes / (dom_ms / dom_n / 1e3) / 1e9 if abytes else None
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None, "traffic": None,
                "algorithmic_bytes_per_launch": abytes, "avg_launch_us": 1e3 * dom_ms / dom_n,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "note": (f"{cg_per_launch:.1f} PCG iterations per launch; the sheet's system "
                         "sits in L2; " + ("one thread block runs the solve" if sc.n_free <= 1024 else
                                            "co-resident blocks with grid barriers run the solve "
                                            "(t2_pcg_grid)"))
                        if dom == "t2_pcg" else None}
    sc.close()
    newton = float(np.mean([t["newton_iterations"] for t in stats]))
    cgits = float(np.mean([t["cg_iterations"] for t in stats]))
    line = {
        "metric": "2-D timesteps/s (tri2d sheet)", "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload, "tris": spec.n_tris, "vertices": spec.n_vertices,
                   "free_dofs": 2 * sc.n_free, "blocks": sc.nnzb, "precision": "fp64",
                   "solver": "eigen-pcg-diag (1e-10)", "l2": "working set < L2 (resident)",
                   "parallelism": f"replicas{ws}"},
        "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
        "wall_ms_per_step": 1000.0 * wall / args.steps,
        "newton_iterations_per_step": newton, "cg_iterations_per_step": cgits,
        "clocks": clocks, "e2e": e2e, "roofline": roof, "gpu_launches": launches,
        "profiled_replay_ms_per_step": float(np.mean(prof_ms)), "kernels": per_kernel,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = tri2d_cpu_baseline(spec, workload, budget_s=20.0,
                                                  max_steps=args.warmup + args.steps,
                                                  threads=args.cpu_threads)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def tri2d_cpu_baseline(spec, workload, budget_s, max_steps, threads=0):
    """The FP64 2-D oracle (OpenMP over the host cores) stepping the same
    sheet from its initial state: seconds per step over a bounded sample."""
    import oracle
    threads = oracle.set_threads(threads or os.cpu_count())
    o = oracle.OracleTri2d(spec)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and (n == 0 or time.perf_counter() - t0 < budget_s):
        o.step()
        n += 1
    t = (time.perf_counter() - t0) / n
    return {"value": 1.0 / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"FP64 2-D oracle on {threads} host threads, {workload}: {n} steps from the "
                      f"initial state, {t:.3f} s per step"}


def run_reference_tri2d(args):
    ws, rank, _, _ = dist_setup()
    if rank != 0:
        return 0
    spec, workload = tri2d_workload(args.sheet)
    cb = tri2d_cpu_baseline(spec, workload, budget_s=120.0, max_steps=args.warmup + args.steps,
                            threads=args.cpu_threads)
    value = cb["value"]
    line = {"impl": "reference", "metric": "2-D timesteps/s (tri2d sheet)", "value": value,
            "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "precision": "fp64"}, "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.config == "tri2d":
        return run_reference_tri2d(args) if args.impl == "reference" else run_tri2d(args)
    if args.impl == "ours" and args.config == "c5":
        return run_served(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
