"""bench.py's tri2d line assembled on the CPU with a stand-in scene (the
bookkeeping of the JSON contract; the GPU numbers come from a GB300)."""
import argparse
import io
import json
import sys
from contextlib import redirect_stdout

import pytest

import bench


class FakeStats:
    def __init__(self, k):
        self.status, self.newton_iterations, self.cg_iterations = 0, 3, 100 + k
        self.device_ms = 2.0 + 0.01 * k

    def as_dict(self):
        return {"status": self.status, "newton_iterations": self.newton_iterations,
                "cg_iterations": self.cg_iterations, "device_ms": self.device_ms}


class FakeScene:
    def __init__(self, spec):
        self.spec, self.n_free, self.nnzb, self._h = spec, spec.n_vertices - 10, 7 * spec.n_vertices, None
        self.k, self.prof = 0, False
        self.ms = {n: 0.0 for n in ("t2_elem", "t2_rows", "t2_norm", "t2_pcg", "t2_local",
                                    "t2_energy", "t2_esum", "t2_apply", "t2_history")}
        self.n = dict.fromkeys(self.ms, 0)

    def step(self):
        self.k += 1
        for name, per in (("t2_elem", 3), ("t2_rows", 3), ("t2_pcg", 3), ("t2_energy", 5)):
            self.n[name] += per
            if self.prof:
                self.ms[name] += per * (1.0 if name == "t2_pcg" else 0.05)
        return FakeStats(self.k)

    def kernel_stats(self):
        return {k: (self.ms[k], self.n[k]) for k in self.ms}

    def set_profiling(self, on):
        self.prof = bool(on)

    def close(self):
        pass


def test_tri2d_line_bookkeeping(monkeypatch):
    import mfem_gb300.build
    import mfem_gb300.tri2d
    import mfem_gb300._lib
    monkeypatch.setattr(mfem_gb300.build, "build", lambda *a, **k: None)
    monkeypatch.setattr(mfem_gb300.tri2d, "Tri2dScene", FakeScene)
    monkeypatch.setattr(mfem_gb300._lib, "load", lambda *a, **k: None)
    args = argparse.Namespace(sheet=16, steps=4, warmup=3, no_e2e=True, no_cpu_baseline=False,
                              cpu_threads=2)
    out = io.StringIO()
    try:
        with redirect_stdout(out):
            assert bench.run_tri2d(args) == 0
    finally:
        import os
        import oracle
        oracle.set_threads(os.cpu_count())
    line = json.loads(out.getvalue().strip().splitlines()[-1])
    assert line["config"]["workload"] == "sheet2d_16x4_128tris"
    assert line["value"] == pytest.approx(4 / (sum(2.0 + 0.01 * k for k in range(4, 8)) / 1e3))
    assert line["gpu_launches"] == 4 * (3 + 3 + 3 + 5)
    roof = line["roofline"]
    assert roof["kernel"] == "t2_pcg" and roof["avg_launch_us"] == pytest.approx(1000.0)
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    assert line["kernels"]["t2_pcg"]["launches"] == 12
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] > 0
