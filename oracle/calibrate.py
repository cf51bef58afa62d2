"""TEST INFRASTRUCTURE ONLY: measures, with the FP64 oracle, how many Newton
iterations per timestep a workload takes at its stopping criterion, so that
the CPU baseline timed per Newton iteration can be stated per timestep.

Writes oracle/calibration.json (per-step Newton and PCG iteration counts from
the first step on).  Run from the repository root:
    python oracle/calibrate.py --steps 23 --sizes 60
"""
import argparse
import json
import os
import sys
import time

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--sizes", default="60")
    args = ap.parse_args()
    import oracle
    from mfem_gb300 import abi, configs
    out_path = os.path.join(ROOT, "oracle", "calibration.json")
    out = json.load(open(out_path)) if os.path.exists(out_path) else {}
    for n in [int(v) for v in args.sizes.split(",")]:
        spec = configs.cube_c2(n=n, precision=abi.PRECISION_FP64)
        sc = oracle.OracleScene(spec)
        its, cgs, secs = [], [], []
        for _ in range(args.steps):
            t = time.perf_counter()
            st = sc.step()
            secs.append(time.perf_counter() - t)
            its.append(st.newton_iterations)
            cgs.append(st.cg_iterations)
            print(n, st.newton_iterations, st.cg_iterations, st.residual / st.residual0, secs[-1], flush=True)
        out[f"c2_{n}"] = {"newton_iterations_per_step": sum(its) / len(its),
                          "cg_iterations_per_step": sum(cgs) / len(cgs),
                          "newton_iterations": its, "cg_iterations": cgs,
                          "steps": args.steps, "threads": oracle.lib().oracle_get_threads(),
                          "seconds_per_step_here": sum(secs) / len(secs),
                          "criterion": "relative residual 1e-5, PCG 1e-4"}
        json.dump(out, open(out_path, "w"), indent=1)


if __name__ == "__main__":
    main()
