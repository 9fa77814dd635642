"""Host-side logic without a GPU: the solve pool's admission, ordering and error
reporting (fake contexts and runners), the serving statistics, and the replica timing
protocol of bench.py over a world_size-2 gloo group."""
import os
import socket
import sys
import time
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from networksolvers_gb300 import batch, models  # noqa: E402


class FakeCtx:
    def synchronize(self):
        pass

    def close(self):
        pass


def _jobs(n, footprint=100, arrivals=None):
    H, psi0 = models.heisenberg_chain(4), models.random_state(models.chain_graph(4), 2, seed=0)
    out = []
    for k in range(n):
        j = batch.dmrg_job(H, psi0, tag=k, arrival=(arrivals[k] if arrivals else 0.0))
        j.footprint = footprint
        out.append(j)
    return out


def test_pool_serialises_jobs_that_do_not_fit_together():
    res = batch.SolvePool(workers=4, hbm_bytes=150, context_factory=FakeCtx,
                          runner=lambda j, c: (time.sleep(0.03), j.tag)[1]).run(_jobs(4))
    spans = sorted((r.start, r.finish) for r in res)
    for (s0, f0), (s1, f1) in zip(spans, spans[1:]):
        assert s1 >= f0 - 1e-6
    assert [r.value for r in res] == [0, 1, 2, 3]


def test_pool_overlaps_jobs_that_fit_and_respects_arrivals():
    arr = [0.0, 0.0, 0.1, 0.1]
    res = batch.SolvePool(workers=4, hbm_bytes=1000, context_factory=FakeCtx,
                          runner=lambda j, c: (time.sleep(0.05), j.tag)[1]).run(_jobs(4, arrivals=arr))
    assert res[1].start < res[0].finish  # the first two overlap
    for r, a in zip(res, arr):
        assert r.start >= a - 1e-3
    assert all(r.error is None for r in res)


def test_pool_reports_failures_and_keeps_serving():
    def runner(j, c):
        if j.tag == 1:
            raise RuntimeError("boom")
        return j.tag

    res = batch.SolvePool(workers=2, hbm_bytes=1000, context_factory=FakeCtx, runner=runner).run(_jobs(4))
    assert res[1].error and "boom" in res[1].error
    assert [r.value for r in res if r.error is None] == [0, 2, 3]
    summ = batch.latency_summary(res)
    assert summ["solves"] == 3 and summ["failed"] == 1


def test_footprint_grows_with_bond_dimension():
    H, psi0 = models.heisenberg_chain(20), models.random_state(models.chain_graph(20), 4, seed=0)
    f = [batch.footprint_bytes(batch.dmrg_job(H, psi0, maxdim=m)) for m in (32, 128, 512)]
    assert f[0] < f[1] < f[2]


def test_poisson_arrivals():
    arr = batch.poisson_arrivals(50.0, 20.0, seed=3)
    assert all(0 <= a < 20.0 for a in arr) and arr == sorted(arr)
    assert abs(len(arr) - 1000) < 5 * np.sqrt(1000)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_rank(rank, world, port, q):
    import torch.distributed as td
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.replica_time(1.0 + rank)  # rank 1 is the slower replica
    q.put((rank, t, bench.replica_throughput(world, 2, t)))
    td.barrier()
    td.destroy_process_group()


def test_replica_timing_over_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]      # both ranks report the slowest replica
    assert all(abs(o[2] - 2.0) < 1e-12 for o in out)  # 2 replicas x 2 steps / 2 s
