"""Concurrent solves (networksolvers_gb300.batch): every result is the same alone and in
the mix, and admission respects the HBM budget."""
import numpy as np
import pytest

from networksolvers_gb300 import batch, models

pytestmark = pytest.mark.gpu


def _mix():
    jobs = []
    for k in range(6):
        n = 10 + 2 * k
        H = models.j1j2_chain(n, 0.1 * k)
        psi0 = models.random_state(models.chain_graph(n), 4, seed=k)
        jobs.append(batch.dmrg_job(H, psi0, tag=("dmrg", k), nsweeps=3, maxdim=16 + 8 * k, cutoff=1e-10))
    g = models.binary_tree_graph(3)
    H = models.tfim_tree(g, h=0.8).astype(np.complex128)
    jobs.append(batch.tdvp_job(H, models.all_up_state(g), [0.05 * i for i in range(1, 5)], tag=("tdvp", 0),
                               maxdim=16))
    return jobs


def test_results_identical_alone_and_in_the_mix():
    alone = batch.SolvePool(workers=1, precision="fp64").run(_mix())
    mixed = batch.SolvePool(workers=4, precision="fp64").run(_mix())
    assert all(r.error is None for r in alone + mixed), [r.error for r in alone + mixed if r.error]
    for a, b in zip(alone, mixed):
        assert a.tag == b.tag
        if a.kind == "dmrg":
            assert a.value == b.value  # bitwise: same kernels in the same order on each solve's stream
        else:
            for v in a.value:
                np.testing.assert_array_equal(a.value[v], b.value[v])
    # the solves did overlap in the mix
    starts = sorted(r.start for r in mixed)
    ends = sorted(r.finish for r in mixed)
    assert starts[1] < ends[0]


def test_admission_by_footprint():
    jobs = _mix()[:4]
    for j in jobs:
        j.footprint = 100
    # budget for one job at a time: the pool must serialise them
    res = batch.SolvePool(workers=4, precision="fp64", hbm_bytes=150).run(jobs)
    spans = sorted((r.start, r.finish) for r in res)
    for (s0, f0), (s1, f1) in zip(spans, spans[1:]):
        assert s1 >= f0 - 1e-6
    assert all(r.error is None for r in res)
