"""Per-phase device timers of the region step (nsg_ctx_timers / nsg_ctx_phase /
nsg_get_timers): a DMRG run through the general driver records one extraction, one
Krylov and one factorization interval per region, H_eff applications inside the Krylov
phase and the density-matrix expansion inside extraction; the fused chain driver records
its phases from inside nsg_region_step; nothing is recorded while the timers are off;
misuse is rejected."""
import pytest

import networksolvers_gb300 as ns
import networksolvers_gb300.models as m
from networksolvers_gb300 import _native
from networksolvers_gb300.chain import dmrg_chain

pytestmark = pytest.mark.gpu

TRUNC = dict(cutoff=1e-10, maxdim=16)


def _run_general(nsweeps=2):
    H, psi0 = m.heisenberg_chain(10), m.random_state(m.chain_graph(10), 4, seed=3)
    regions = []
    ns.dmrg(H, psi0, nsweeps=nsweeps, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
            extracter_kwargs=dict(trunc=TRUNC, subspace_algorithm="densitymatrix"), inserter_kwargs=dict(trunc=TRUNC),
            region_callback=lambda *a, **k: regions.append(1))
    return len(regions)


def test_phase_timers_general_driver(nsg_ctx):
    nsg_ctx.timers(True)
    try:
        regions = _run_general()
        t = nsg_ctx.read_timers()
    finally:
        nsg_ctx.timers(False)
    for ph in ("extract", "krylov", "factorize"):
        assert t[ph]["count"] == regions and t[ph]["ms"] > 0, (ph, t[ph], regions)
    assert t["heff"]["count"] >= regions and 0 < t["heff"]["ms"] < t["krylov"]["ms"], t
    assert 0 < t["subspace"]["count"] <= regions and 0 < t["subspace"]["ms"] < t["extract"]["ms"], t
    # off: nothing is recorded
    _run_general(nsweeps=1)
    assert all(v["count"] == 0 and v["ms"] == 0 for v in nsg_ctx.read_timers().values())


def test_phase_timers_fused_chain_driver(nsg_ctx):
    H, psi0 = m.heisenberg_chain(12), m.random_state(m.chain_graph(12), 4, seed=5)
    nsg_ctx.timers(True)
    try:
        E, _, records = dmrg_chain(H, psi0, 2, maxdim=16, cutoff=1e-10, ctx=nsg_ctx)
        t = nsg_ctx.read_timers()
    finally:
        nsg_ctx.timers(False)
    regions = len(records)
    for ph in ("extract", "krylov", "factorize"):
        assert t[ph]["count"] == regions and t[ph]["ms"] > 0, (ph, t[ph], regions)
    assert t["heff"]["count"] >= regions and t["heff"]["ms"] < t["krylov"]["ms"]
    assert t["subspace"]["count"] == 0


def test_phase_misuse_is_rejected(nsg_ctx):
    L = nsg_ctx.L
    assert L.nsg_ctx_phase(nsg_ctx.h, 5, 1) == _native.ERR_INVALID
    assert L.nsg_ctx_phase(nsg_ctx.h, -1, 0) == _native.ERR_INVALID
    nsg_ctx.timers(True)
    try:
        assert L.nsg_ctx_phase(nsg_ctx.h, 0, 0) == _native.ERR_INVALID  # not open
        assert L.nsg_ctx_phase(nsg_ctx.h, 0, 1) == _native.OK
        assert L.nsg_ctx_phase(nsg_ctx.h, 0, 1) == _native.ERR_INVALID  # already open
        assert L.nsg_ctx_phase(nsg_ctx.h, 0, 0) == _native.OK
        assert nsg_ctx.read_timers()["extract"]["count"] == 1
    finally:
        nsg_ctx.timers(False)
