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
  e2e         the same metric through the C ABI with host buffers: every step
              uploads the pinned positions from host memory and reads the new
              vertex positions back
  roofline    the dominant kernel's algorithmic bytes per launch / its average
              launch time (CUDA events around every launch in the timed steps)
  cpu_baseline  the FP64 oracle port on the host cores, one Newton iteration of
              the same scene (bounded sample), scaled by Newton iterations/step
  --impl reference  the same oracle port as the reference's CPU arm.

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
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4"])
    ap.add_argument("--size", type=int, default=60, help="cubes per axis for c2")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--solver", default="eigen-pcg-diag", choices=["eigen-pcg-diag", "gpu-pcg-block"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-threads", type=int, default=0)
    return ap.parse_args()


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
def kernel_bytes(kind, sizes, rsz):
    """Algorithmic bytes per launch (each array read or written once)."""
    nt, nv, nf, nnzb, n_inc, nnz_m = (sizes[k] for k in ("nt", "nv", "nf", "nnzb", "n_inc", "nnz_m"))
    if kind == "k_cg_spmv":
        # values + block cols + row ptr, z and p_prev read, Ap and p written
        return nnzb * (9 * rsz + 4) + 4 * (nf + 1) + 4 * 3 * nf * rsz
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
    return None


def read_traffic(kernel, workload):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
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
    solver = abi.SOLVER_EIGEN_CG_DIAG if args.solver == "eigen-pcg-diag" else abi.SOLVER_GPU_PCG_BLOCK
    if args.config == "c1":
        return configs.beam_c1(precision=prec, linear_solver=solver), "beam_c1_200tets"
    if args.config == "c3":
        return configs.stress_c3(precision=prec, linear_solver=solver), "stress_c3_135k"
    n = args.size
    return configs.cube_c2(n=n, precision=prec, linear_solver=solver), f"cube_c2_{n}^3_{5 * n ** 3}tets"


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


# ------------------------------------------------------------ CPU sample --
def cpu_newton_sample(spec, threads):
    """FP64 oracle: seconds of one Newton iteration of the scene (update,
    assembly, PCG to the scene's tolerance, local solve, line search)."""
    import copy
    import oracle
    oracle.set_threads(threads)
    s = copy.copy(spec)
    s.max_newton_iterations = 1
    sc = oracle.OracleScene(s)
    t0 = time.perf_counter()
    st = sc.step()
    t1 = time.perf_counter()
    return t1 - t0, st


def run_reference(args):
    ws, rank, _, pg = dist_setup()
    if rank != 0:
        return 0
    import oracle  # noqa: F401  (the reference arm is the FP64 port on the host cores)
    from mfem_gb300 import abi
    threads = args.cpu_threads or os.cpu_count()
    spec, workload = make_spec(args, "fp64")
    iters_per_step = _newton_iters_hint(args)
    times = []
    for i in range(args.warmup + args.steps):
        t, st = cpu_newton_sample(spec, threads)
        if i >= args.warmup:
            times.append(t)
    t_iter = float(np.mean(times))
    value = 1.0 / (t_iter * iters_per_step)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": workload, "precision": "fp64",
                                        "solver": args.solver},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"one Newton iteration of {workload} per step "
                                   f"({t_iter:.2f} s), x {iters_per_step} Newton iterations/step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _newton_iters_hint(args):
    """Newton iterations per step of this workload at the 1e-5 residual test
    (measured by the oracle, oracle/calibration.json), default 4."""
    p = os.path.join(ROOT, "oracle", "calibration.json")
    if os.path.exists(p):
        d = json.load(open(p))
        key = f"{args.config}_{args.size}" if args.config == "c2" else args.config
        if key in d:
            return float(d[key]["newton_iterations_per_step"])
    return 4.0


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
    barrier(pg)
    gpu.set_profiling(batch_h, True)
    sampler = ClockSampler(local)
    sampler.start()
    ms, stats = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = scene.step()
        ms.append(st.device_ms)
        stats.append(st.as_dict())
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    kstats = gpu.kernel_stats(batch_h)
    gpu.set_profiling(batch_h, False)
    dev_s = sum(ms) / 1000.0
    dev_s_max = allmax(pg, dev_s)
    value = ws * args.steps / dev_s_max

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        pins = scene.pinned()
        state = scene.get_state()
        pin_host = np.ascontiguousarray(state["x"][pins])
        x_host = np.zeros((scene.n_vertices, 3))
        n_e2e = max(3, args.steps // 2)
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            scene.set_pins(pin_host)                       # H2D: this step's pinned targets
            scene.step()
            L.mfem_gpu_scene_get_state(scene.handle, x_host.ctypes.data_as(
                ctypes.POINTER(ctypes.c_double)), None, None, None, None)  # D2H: positions
        e2e_s = allmax(pg, time.perf_counter() - t0)
        e2e = {"value": ws * n_e2e / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(pin_host.nbytes), "d2h_bytes_per_step": int(x_host.nbytes),
               "steps": n_e2e}

    # ---- roofline of the dominant kernel
    dom = max(kstats, key=lambda k: kstats[k][0])
    dom_ms, dom_n = kstats[dom]
    abytes = kernel_bytes(dom, sizes, rsz)
    peak, peak_src = measured_peak()
    achieved = abytes / (dom_ms / dom_n / 1e3) / 1e9 if abytes and dom_n else None
    roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "traffic": read_traffic(dom, "c2"),
            "algorithmic_bytes_per_launch": abytes, "avg_launch_us": 1e3 * dom_ms / dom_n,
            "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"}
    per_kernel = {}
    for k, (kms, kn) in kstats.items():
        if kn:
            b = kernel_bytes(k, sizes, rsz)
            per_kernel[k] = {"ms": round(kms, 3), "launches": kn,
                             "share": round(kms / max(dev_s * 1e3, 1e-9), 4),
                             "GBps": round(b / (kms / kn / 1e3) / 1e9, 1) if (b and kms > 0) else None}
    launches = int(sum(n for (_, n) in kstats.values()))

    newton = float(np.mean([s["newton_iterations"] for s in stats]))
    cgits = float(np.mean([s["cg_iterations"] for s in stats]))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": workload, "tets": sizes["nt"], "vertices": sizes["nv"],
                   "free_dofs": 3 * sizes["nf"], "blocks": sizes["nnzb"],
                   "precision": args.precision, "solver": args.solver,
                   "newton_residual_tolerance": spec.newton_residual_tolerance,
                   "pcg_tolerance": spec.iterative_solver_tolerance,
                   "l2": "working set > L2 (about 1 GB per step)",
                   "parallelism": f"replicas{ws}"},
        "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
        "wall_ms_per_step": 1000.0 * wall / args.steps,
        "newton_iterations_per_step": newton, "cg_iterations_per_step": cgits,
        "residual_rel_last": stats[-1]["residual"] / max(stats[-1]["residual0"], 1e-300),
        "clocks": clocks, "e2e": e2e, "roofline": roof, "gpu_launches": launches,
        "kernels": per_kernel,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = args.cpu_threads or os.cpu_count()
        ref_spec, _ = make_spec(args, "fp64")
        t_it, _ = cpu_newton_sample(ref_spec, threads)
        cpu_val = 1.0 / (t_it * newton)
        line["cpu_baseline"] = {"value": cpu_val, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"one FP64 Newton iteration of {workload} "
                                          f"({t_it:.2f} s) x {newton:.2f} Newton iterations/step"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    scene.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
