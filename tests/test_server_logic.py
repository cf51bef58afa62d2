"""Admission and batching logic of the serving loop, with fake scenes (no GPU)."""
import numpy as np

from mfem_gb300 import abi, server


class _Stats:
    def __init__(self):
        self.device_ms = 1.0
        self.newton_iterations = 2
        self.cg_iterations = 10
        self.status = abi.OK


class _FakeGpu:
    def __init__(self):
        self.batches = []
        self.live = set()

    def footprint(self, spec):
        return spec["bytes"]

    def Scene(self, spec):
        gpu = self

        class S:
            def __init__(self):
                self.spec = spec
                self.x = np.zeros((1, 3))
                gpu.live.add(spec["name"])

            def get_state(self):
                return {"x": self.x.copy()}

            def close(self):
                gpu.live.discard(spec["name"])
        return S()

    def Batch(self, scenes):
        gpu = self
        names = tuple(s.spec["name"] for s in scenes)
        gpu.batches.append(names)
        used = sum(s.spec["bytes"] for s in scenes)

        class B:
            def step(self, raise_on_error=True):
                assert used <= 100
                for s in scenes:
                    s.x += 1.0
                return [_Stats() for _ in scenes]

            def close(self):
                pass
        return B()


def test_admission_by_budget_and_leaving_batches(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=100)
    specs = [dict(name="a", bytes=60), dict(name="b", bytes=30), dict(name="c", bytes=50),
             dict(name="d", bytes=10)]
    steps = [3, 1, 2, 2]
    for sp, n in zip(specs, steps):
        srv.submit(sp, n)
    out = srv.run(realtime=False)
    # every request took its own number of steps, and its state shows it
    for r, n in zip(out, steps):
        assert r.steps_done == n and r.result["x"][0, 0] == n
    # the budget held at every tick (asserted in the fake) and nothing leaked
    assert not fake.live
    # c waited for memory: it only joined after a and b left
    first_c = next(i for i, b in enumerate(fake.batches) if "c" in b)
    assert all("a" not in b for b in fake.batches[first_c:])
    s = server.summary(out, srv.ticks, 1.0)
    assert s["timesteps"] == sum(steps) and s["requests"] == 4


def test_oversize_request_is_refused(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=10)
    try:
        srv.submit(dict(name="big", bytes=11), 1)
    except ValueError:
        return
    raise AssertionError("oversize request accepted")
