"""The N > 1 path on CPU: two gloo ranks (bench.py's process-group helpers)
share a served stream by server.shard, each serving its part with no
exchange, and agree on the whole-job figures."""
import multiprocessing as mp
import os
import socket
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Stats:
    def __init__(self):
        self.device_ms, self.newton_iterations, self.cg_iterations, self.status = 1.0, 2, 10, 0


class _FakeGpu:
    """Scenes whose x counts their steps; no device."""

    def footprint(self, spec):
        return spec.bytes

    def Scene(self, spec):
        class S:
            def __init__(self):
                self.spec, self.x = spec, np.zeros((1, 3))

            def get_state(self):
                return {"x": self.x.copy()}

            def checkpoint(self):
                pass

            def close(self):
                pass
        return S()

    def Batch(self, scenes):
        class B:
            def step(self, raise_on_error=True):
                for s in scenes:
                    s.x += 1.0
                return [_Stats() for _ in scenes]

            def close(self):
                pass
        return B()


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from mfem_gb300 import abi, server
    server.gpu = _FakeGpu()
    ws, r, _, pg = bench.dist_setup()
    weights = [5, 1, 4, 4, 2, 7, 3]           # tets x steps of seven requests
    mine = server.shard(weights, ws, r)
    srv = server.Server(budget_bytes=100, steps_per_tick=1)
    for i in mine:
        srv.submit(SimpleNamespace(bytes=10, precision=abi.PRECISION_MIXED), weights[i])
    out = srv.run(realtime=False)
    steps = sum(o.steps_done for o in out)
    q.put((r, ws, mine, bench.allsum(pg, steps), bench.allmax(pg, float(r + 1)),
           all(o.result["x"][0, 0] == o.steps for o in out)))
    bench.barrier(pg)
    pg.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_share_a_stream():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, m0, tot0, mx0, ok0), (r1, ws1, m1, tot1, mx1, ok1) = res
    assert (r0, r1, ws0, ws1) == (0, 1, 2, 2)
    assert sorted(m0 + m1) == list(range(7)) and not set(m0) & set(m1)
    assert tot0 == tot1 == 26.0 and mx0 == mx1 == 2.0 and ok0 and ok1
    # greedy by weight: 7 | 5 | 4 -> 5 | 4 -> 7 ... balanced to 13 / 13
    w = [5, 1, 4, 4, 2, 7, 3]
    assert sum(w[i] for i in m0) == sum(w[i] for i in m1) == 13


def test_shard_single_rank_takes_all():
    sys.path.insert(0, ROOT)
    from mfem_gb300 import server
    assert server.shard([3, 1, 2], 1, 0) == [0, 1, 2]
    assert server.shard([], 4, 2) == []
