"""Admission, batching and precision escalation of the serving loop, with
fake scenes (no GPU)."""
from types import SimpleNamespace

import numpy as np

from mfem_gb300 import abi, server


def _spec(name, nbytes, precision=abi.PRECISION_MIXED, ls_fail_at=None, fail=abi.ERR_LS_FAILED):
    return SimpleNamespace(name=name, bytes=nbytes, precision=precision, ls_fail_at=ls_fail_at,
                           fail=fail)


class _Stats:
    def __init__(self, status=abi.OK):
        self.device_ms = 1.0
        self.newton_iterations = 2
        self.cg_iterations = 10
        self.status = status


class _FakeGpu:
    """Scenes carry a step counter in x; an FP64 scene needs twice the bytes.
    A mixed scene with ls_fail_at reports a failed line search at that step."""

    def __init__(self):
        self.batches = []
        self.live = set()

    def footprint(self, spec):
        return spec.bytes * (2 if spec.precision == abi.PRECISION_FP64 else 1)

    def Scene(self, spec):
        gpu = self

        class S:
            def __init__(self):
                self.spec = spec
                self.x = np.zeros((1, 3))
                self.key = (spec.name, spec.precision)
                assert self.key not in gpu.live
                gpu.live.add(self.key)

            def get_state(self):
                z = np.zeros(1)
                return {"x": self.x.copy(), "v": z, "s": z, "R": z}

            def checkpoint(self):
                self.saved = self.x.copy()

            def rollback(self):
                self.x = self.saved.copy()

            def snapshot(self):
                return self.x.tobytes()

            def restore(self, snap):
                self.x = np.frombuffer(snap, dtype=float).reshape(1, 3).copy()

            def close(self):
                gpu.live.discard(self.key)
        return S()

    def Batch(self, scenes):
        gpu = self
        assert len({s.spec.precision for s in scenes}) == 1
        names = tuple(s.spec.name for s in scenes)
        gpu.batches.append((scenes[0].spec.precision, names))

        class B:
            def step(self, raise_on_error=True):
                used = sum(gpu.footprint(s.spec) for s in scenes if s.key in gpu.live)
                assert all(s.key in gpu.live for s in scenes)
                assert used <= 200
                out = []
                for s in scenes:
                    s.x += 1.0
                    fail = (s.spec.precision == abi.PRECISION_MIXED
                            and s.spec.ls_fail_at == int(s.x[0, 0]))
                    out.append(_Stats(s.spec.fail if fail else abi.OK))
                return out

            def step_n(self, k, raise_on_error=True):
                # k steps per scene; a scene's status is the worst of its steps
                worst = [abi.OK] * len(scenes)
                done = np.zeros((len(scenes), k))
                for j in range(k):
                    for i, st in enumerate(self.step()):
                        if st.status != abi.OK:
                            worst[i] = st.status
                        done[i, j] = j + 1.0
                return [_Stats(w) for w in worst], done

            def close(self):
                pass
        return B()


def test_admission_by_budget_and_leaving_batches(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=100, steps_per_tick=1)
    specs = [_spec("a", 60), _spec("b", 30), _spec("c", 50), _spec("d", 10)]
    steps = [3, 1, 2, 2]
    for sp, n in zip(specs, steps):
        srv.submit(sp, n)
    out = srv.run(realtime=False)
    # every request took its own number of steps, and its state shows it
    for r, n in zip(out, steps):
        assert r.steps_done == n and r.result["x"][0, 0] == n and r.escalated_at is None
    # nothing leaked
    assert not fake.live
    # c waited for memory: it only joined after a and b left
    first_c = next(i for i, (_, b) in enumerate(fake.batches) if "c" in b)
    assert all("a" not in b for _, b in fake.batches[first_c:])
    s = server.summary(out, srv.ticks, 1.0)
    assert s["timesteps"] == sum(steps) and s["requests"] == 4 and s["escalated_to_fp64"] == 0


def test_failed_line_search_continues_in_fp64(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=200, steps_per_tick=1)
    srv.submit(_spec("soft", 40, ls_fail_at=2), 5)
    srv.submit(_spec("stiff", 40), 4)
    srv.submit(_spec("last", 40, ls_fail_at=3), 3)   # fails on its final step
    srv.submit(_spec("rot", 20, ls_fail_at=1, fail=abi.ERR_PROCRUSTES), 2)
    out = srv.run(realtime=False)
    soft, stiff, last, rot = out
    # the failed step is rolled back and taken again in FP64
    assert soft.escalated_at == 1 and soft.steps_done == 5 and soft.result["x"][0, 0] == 5
    assert len(soft.newton) == 5 and soft.footprint == 80
    assert last.escalated_at == 2 and last.result["x"][0, 0] == 3
    assert rot.escalated_at == 0 and rot.status == abi.OK and rot.result["x"][0, 0] == 2
    assert stiff.escalated_at is None
    # after the failure the two precisions ran as two batches in the same ticks
    precs = [p for p, names in fake.batches if "soft" in names]
    assert precs[0] == abi.PRECISION_MIXED and precs[-1] == abi.PRECISION_FP64
    assert any(p == abi.PRECISION_MIXED and "stiff" in names for p, names in fake.batches[-2:])
    assert not fake.live
    s = server.summary(out, srv.ticks, 1.0)
    assert s["escalated_to_fp64"] == 3 and s["failed_requests"] == 0


def test_escalation_off_keeps_mixed(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=200, escalate=False, steps_per_tick=1)
    srv.submit(_spec("soft", 40, ls_fail_at=2), 4)
    (r,) = srv.run(realtime=False)
    assert r.escalated_at is None and r.steps_done == 4
    assert all(p == abi.PRECISION_MIXED for p, _ in fake.batches)


def test_oversize_request_is_refused(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=10)
    try:
        srv.submit(_spec("big", 11), 1)
    except ValueError:
        return
    raise AssertionError("oversize request accepted")


def test_empty_stream_and_bad_requests(monkeypatch):
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=100)
    assert srv.run(realtime=False) == []
    for bad in (0, -3):
        try:
            srv.submit(_spec("z", 10), bad)
        except ValueError:
            continue
        raise AssertionError("a request without timesteps was accepted")
    s = server.summary([], [], 1.0)
    assert s["timesteps"] == 0 and s["requests"] == 0


def test_shard_is_balanced_and_deterministic():
    w = [9, 1, 8, 2, 7, 3, 6, 4, 5]
    parts = [server.shard(w, 3, r) for r in range(3)]
    assert sorted(i for p in parts for i in p) == list(range(9))
    loads = [sum(w[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(w)
    assert parts == [server.shard(w, 3, r) for r in range(3)]


def test_lane_partition_balances_by_weight():
    from mfem_gb300 import gpu
    w = [100, 5, 60, 40, 35, 30, 1, 9]
    parts = gpu.lane_partition(w, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(w)))
    loads = [sum(w[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(w)
    assert parts == gpu.lane_partition(w, 3)
    assert gpu.lane_partition([3, 2], 5) == [[0], [1]]


def test_multi_step_ticks_roll_back_the_whole_tick(monkeypatch):
    """Ticks of several timesteps (each scene at its own pace): a tick never
    takes a scene past its own count, and a failed step rolls the scene back
    to the tick's start, from where the FP64 scene takes the tick again."""
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=200, steps_per_tick=4)
    srv.submit(_spec("soft", 40, ls_fail_at=6), 9)
    srv.submit(_spec("stiff", 40), 10)
    out = srv.run(realtime=False)
    soft, stiff = out
    # ticks of min(4, what the members still owe): 4, 4, then 1 for soft
    assert soft.escalated_at == 4 and soft.steps_done == 9 and soft.result["x"][0, 0] == 9
    assert stiff.escalated_at is None and stiff.steps_done == 10 and stiff.result["x"][0, 0] == 10
    assert len(soft.step_ms) == 9 and len(stiff.step_ms) == 10
    assert not fake.live


def test_lanes_serve_every_request_in_its_own_loop(monkeypatch):
    """lanes > 1: requests dealt out by work to independent loops (own
    batches, own thread, budget / lanes each); every request still takes
    exactly its timesteps, escalation still works, nothing leaks."""
    fake = _FakeGpu()
    monkeypatch.setattr(server, "gpu", fake)
    srv = server.Server(budget_bytes=200, lanes=2)
    reqs = [("a", 40, 3, None), ("b", 30, 5, None), ("c", 20, 2, 1), ("d", 40, 4, None), ("e", 10, 6, None)]
    for name, nb, n, fail in reqs:
        srv.submit(_spec(name, nb, ls_fail_at=fail), n)
    out = srv.run(realtime=False)
    for r, (_, _, n, fail) in zip(out, reqs):
        assert r.steps_done == n and r.result["x"][0, 0] == n
        assert (r.escalated_at is not None) == (fail is not None)
    assert not fake.live
    # the greedy deal by footprint x timesteps: a(120) b(150) c(40) d(160) e(60)
    # -> lane 0 a, c, e; lane 1 b, d; no batch mixes the two lanes' requests
    lanes = [{"a", "c", "e"}, {"b", "d"}]
    for _, b in fake.batches:
        assert any(set(b) <= lane for lane in lanes), b
    assert len(srv.ticks) > 0
    try:
        server.Server(budget_bytes=100, lanes=4).submit(_spec("big", 30), 1)
        srv2 = server.Server(budget_bytes=100, lanes=4)
        srv2.submit(_spec("big", 30), 1)
        srv2.run(realtime=False)
    except ValueError:
        return
    raise AssertionError("a request over a lane's budget was accepted")
