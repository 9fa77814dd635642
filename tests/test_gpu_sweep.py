"""Whole-sweep parity on the GPU against the oracle and the golden fixtures.
Tolerances (from the workload definition): energies 1e-10 relative, overlaps and
fidelities 1e-8, truncated bond dimensions exactly equal."""
from pathlib import Path

import numpy as np
import pytest

import networksolvers_gb300 as ns
import networksolvers_gb300.models as m
from networksolvers_gb300 import network as pn

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def test_c1_heisenberg_n20_matches_golden(nsg_ctx):
    gold = np.load(GOLD / "c1_heisenberg_n20.npz")
    H, psi0 = m.config_heisenberg_chain(20, 10, 0)
    rec = []

    def cb(prob, sweep, region, which, **k):
        rec.append((sweep, which, prob.eigenvalue, prob.last_insert.get("newdim", -1)))

    E, psi = ns.dmrg(H, psi0, nsweeps=5, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
                     inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=64)), region_callback=cb)
    rec = np.array(rec)
    assert np.array_equal(rec[:, 3], gold["newdim"]), "truncated bond dimensions differ"
    assert np.max(np.abs(rec[:, 2] - gold["eigenvalue"]) / np.abs(gold["eigenvalue"])) < 1e-10
    assert abs(E - float(gold["energy"])) / abs(float(gold["energy"])) < 1e-10
    assert abs(E - float(gold["ed_energy"])) < 1e-8
    dims = psi.linkdims()
    assert [dims[e] for e in H.graph.edges] == list(gold["linkdims"])


def test_reference_tree_dmrg(nsg_ctx):
    """test_tree_dmrg.jl:13-68 on the GPU: |E - E_ED| < 1e-5 for 2-site and for
    1-site + densitymatrix expansion; parity with the oracle at 1e-10."""
    gold = np.load(GOLD / "tree_dmrg.npz")
    g = m.build_tree_graph(3, 3)
    H, p0 = m.heisenberg_tree(g), m.neel_state(g)
    trunc = dict(cutoff=1e-5, maxdim=40)
    E2, _ = ns.dmrg(H, p0, nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=trunc))
    assert abs(E2 - float(gold["ed_energy"])) < 1e-5
    assert abs(E2 - float(gold["e2"])) < 1e-10 * abs(E2)
    E1, _ = ns.dmrg(H, p0, nsweeps=5, nsites=1, extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
                    inserter_kwargs=dict(trunc=trunc))
    assert abs(E1 - float(gold["ed_energy"])) < 1e-5
    assert abs(E1 - float(gold["e1"])) < 1e-10 * abs(E1)


def _oracle_tdvp(H, psi0, times, nsites, solver):
    from oracle import sweep as osw
    uk = {} if solver == "rk4" else dict(solver=osw.exponentiate_solver)
    return osw.tdvp(H, psi0, times, nsites=nsites, updater_kwargs=uk,
                    inserter_kwargs=dict(trunc=dict(cutoff=1e-9, maxdim=64)))


def _to_oracle(psi_dev, net_like):
    from oracle import network as on
    from networksolvers_gb300.models import Network
    arrs = psi_dev.to_numpy(net_like)
    return Network(net_like.graph, arrs, net_like.legs, np.complex128, {"kind": "state"})


@pytest.mark.parametrize("nsites,solver", [(2, "expo"), (1, "rk4"), (2, "rk4")])
def test_tfim_tree_tdvp_matches_oracle(nsg_ctx, nsites, solver):
    """2-site/1-site TDVP, TFIM on a depth-2 binary tree from the all-up state:
    fidelity with the oracle's state >= 1 - 1e-8."""
    from oracle import network as on
    g = m.binary_tree_graph(2)
    H, psi0 = m.tfim_tree(g, h=1.0).astype(np.complex128), m.all_up_state(g)
    times = [0.0, 0.05, 0.10, 0.15]
    uk = {} if solver == "rk4" else dict(solver=ns.exponentiate_solver)
    psi = ns.tdvp(H, psi0, times, nsites=nsites, updater_kwargs=uk,
                  inserter_kwargs=dict(trunc=dict(cutoff=1e-9, maxdim=64)))
    ref = _oracle_tdvp(H, psi0, times, nsites, solver)
    got, _ = on.from_network(_to_oracle(psi, psi0), site_index={v: [i for i in ref[v].inds if i.tags.startswith("Site")][0]
                                                                 for v in ref.g.vertices})
    f = abs(on.inner(ref, got)) / (ref.norm() * got.norm())
    assert f > 1 - 1e-8


def test_tdvp_exact_evolution(nsg_ctx):
    """2-site TDVP with exponentiate on a 7-site TFIM tree vs exact exp(-iHt)|ψ0>."""
    from oracle import ed
    g = m.binary_tree_graph(2)
    H, psi0 = m.tfim_tree(g, h=1.0).astype(np.complex128), m.all_up_state(g)
    times = np.arange(0, 0.2 + 1e-9, 0.05)
    psi = ns.tdvp(H, psi0, times, nsites=2, updater_kwargs=dict(solver=ns.exponentiate_solver),
                  inserter_kwargs=dict(trunc=dict(cutoff=1e-12, maxdim=64)))
    terms = [(u, v, -1.0, m.PZ, m.PZ) for (u, v) in g.edges]
    Hx = ed.hamiltonian(g.vertices, terms, {v: -1.0 * m.PX for v in g.vertices})
    v0 = np.zeros(2 ** len(g.vertices), complex)
    v0[0] = 1.0
    vt = ed.evolve(Hx, v0, times[-1])
    # contract the device state to a dense vector
    from networksolvers_gb300.itensors import contract
    full = contract([psi[v] for v in psi.g.vertices])
    dense = full.permute([psi.siteind(v) for v in g.vertices]).to_numpy().reshape(-1)
    fid = abs(np.vdot(vt, dense)) / np.linalg.norm(dense)
    assert fid > 1 - 1e-8


def _record_dmrg(run, H, psi0, **kw):
    rec = []

    def cb(prob, sweep, region, which, **k):
        rec.append((sweep, which, prob.eigenvalue, prob.last_insert.get("newdim", -1)))

    E, psi = run(H, psi0, region_callback=cb, **kw)
    return E, np.array(rec), psi


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_c3_style_schedule_with_densitymatrix(nsg_ctx, precision):
    """The large-DMRG recipe at reduced size: Heisenberg N=30, random MPS chi=8 seed 1,
    maxdim schedule [8, 16, 32], cutoff 1e-12, densitymatrix expansion, 2-site.
    FP64: per-region energies 1e-10 and bond dimensions exact vs the oracle.
    TF32x3 (FP32-accumulated contractions): final energy within 1e-5 relative — the
    environments carry the accumulated left/right energies, so 24-bit accumulation
    limits the absolute error of H_eff x to ~5e-7 |E|."""
    from oracle import sweep as osw
    H, psi0 = m.heisenberg_chain(30), m.random_state(m.chain_graph(30), 8, seed=1)
    trunc = dict(cutoff=1e-12, maxdim=[8, 16, 32])
    kw = dict(nsweeps=4, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
              extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
              inserter_kwargs=dict(trunc=trunc))
    Eo, ro, _ = _record_dmrg(osw.dmrg, H, psi0, **kw)
    nsg_ctx.set_precision(precision)
    try:
        E, r, psi = _record_dmrg(ns.dmrg, H, psi0, **kw)
    finally:
        nsg_ctx.set_precision("fp64")
    if precision == "fp64":
        assert np.array_equal(r[:, 3], ro[:, 3])
        assert np.max(np.abs(r[:, 2] - ro[:, 2]) / np.abs(ro[:, 2])) < 1e-10
    assert abs(E - Eo) / abs(Eo) < (1e-10 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("model", ["j1j2", "xxz"])
def test_batch_and_serve_chains_match_oracle(nsg_ctx, model, precision):
    """The chain families of the batched and served workloads (J1-J2 with its w=8 MPO,
    XXZ at anisotropy 1.7) against the oracle: per-region energies 1e-10 relative and
    identical truncated bond dimensions, in the plain and the split form."""
    from oracle import sweep as osw
    n = 14
    H = m.j1j2_chain(n, 0.35) if model == "j1j2" else m.xxz_chain(n, 1.7)
    psi0 = m.random_state(m.chain_graph(n), 8, seed=3)
    kw = dict(nsweeps=3, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
              inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=32)))
    got, ref = [], []

    def cb_got(prob, sweep, region, which, **k):
        got.append((prob.eigenvalue, prob.last_insert.get("newdim", -1)))

    def cb_ref(prob, sweep, region, which, **k):
        ref.append((prob.eigenvalue, prob.last_insert.get("newdim", -1)))

    nsg_ctx.set_precision(precision)
    try:
        E, _ = ns.dmrg(H, psi0, region_callback=cb_got, **kw)
    finally:
        nsg_ctx.set_precision("fp64")
    Eo, _ = osw.dmrg(H, psi0, region_callback=cb_ref, **kw)
    got, ref = np.array(got), np.array(ref)
    assert np.array_equal(got[:, 1], ref[:, 1])
    assert np.max(np.abs(got[:, 0] - ref[:, 0]) / np.abs(ref[:, 0])) < 1e-10
    assert abs(E - Eo) / abs(Eo) < 1e-10


def test_split_form_tracks_plain_form_region_by_region(nsg_ctx):
    """The split form (six-slice tensor-core products; eight-slice in the eigensolver and
    the expansion) against the plain form along the same sweep: Heisenberg N=24, random MPS
    chi=16 seed 1, maxdim schedule [32, 64, 128], cutoff 1e-12, densitymatrix expansion.
    Per-region energies within 1e-10 relative and identical truncated bond dimensions."""
    H, psi0 = m.heisenberg_chain(24), m.random_state(m.chain_graph(24), 16, seed=1)
    trunc = dict(cutoff=1e-12, maxdim=[32, 64, 128])
    kw = dict(nsweeps=3, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
              extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
              inserter_kwargs=dict(trunc=trunc))
    Ep, rp, _ = _record_dmrg(ns.dmrg, H, psi0, **kw)
    nsg_ctx.set_precision("ozaki")
    nsg_ctx.profile(True)
    try:
        Es, rs, _ = _record_dmrg(ns.dmrg, H, psi0, **kw)
        tc = nsg_ctx.profile_read()["tc_gemm"]["launches"]
    finally:
        nsg_ctx.profile(False)
        nsg_ctx.set_precision("fp64")
    assert tc > 0  # the tensor-core products did run
    assert np.array_equal(rs[:, 3], rp[:, 3])
    assert np.max(np.abs(rs[:, 2] - rp[:, 2]) / np.abs(rp[:, 2])) < 1e-10
    assert abs(Es - Ep) / abs(Ep) < 1e-10


def test_opsum_hamiltonian_dmrg_matches_oracle(nsg_ctx):
    """A Hamiltonian written as an OpSum (next-nearest-neighbour exchange, a transverse
    field, a three-site term) compiled to a chain MPO, through the GPU drivers and the
    oracle: per-region energies 1e-10 relative and identical bond dimensions."""
    from oracle import sweep as osw
    n = 12
    os_ = m.OpSum()
    for j in range(1, n):
        os_ += (1.0, "Sz", j, "Sz", j + 1)
        os_ += (0.5, "S+", j, "S-", j + 1)
        os_ += (0.5, "S-", j, "S+", j + 1)
    for j in range(1, n - 1):
        os_ += (0.25, "Sz", j, "Sz", j + 2)
        os_ += (0.1, "Sx", j, "Sz", j + 1, "Sx", j + 2)
    for j in range(1, n + 1):
        os_ += (0.3, "Sx", j)
    H = m.chain_mpo(os_, n)
    psi0 = m.random_state(m.chain_graph(n), 8, seed=2)
    kw = dict(nsweeps=3, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
              inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=32)))
    E, r, _ = _record_dmrg(ns.dmrg, H, psi0, **kw)
    Eo, ro, _ = _record_dmrg(osw.dmrg, H, psi0, **kw)
    assert np.array_equal(r[:, 3], ro[:, 3])
    assert np.max(np.abs(r[:, 2] - ro[:, 2]) / np.abs(ro[:, 2])) < 1e-10
    assert abs(E - Eo) / abs(Eo) < 1e-10


@pytest.mark.parametrize("nsites", [1, 2])
def test_tree_dmrg_with_jumping_post_order_plan(nsg_ctx, nsites):
    """Environment-cache bookkeeping on a tree when consecutive regions are not adjacent:
    DMRG sweeps that follow the post-order DFS plan (dfs_plans.jl:5-16; each move to the
    next region is a gauge walk over several edges and invalidates the environments on
    the way) on the GPU and in the oracle — per-region energies 1e-10 and bond dimensions
    equal."""
    from oracle import network as on, sweep as osw
    g = m.build_tree_graph(3, 2)
    H = m.heisenberg_tree(g)
    psi0 = m.random_state(g, 4, seed=5)
    trunc = dict(cutoff=1e-10, maxdim=16)
    kws = dict(updater_kwargs=dict(krylovdim=3, maxiter=1), inserter_kwargs=dict(trunc=trunc))
    from networksolvers_gb300.sweep import EigsolveProblem, _prepare, sweep_solve, updater_eigsolve

    def run(mod, prep, Problem, solve, upd, plan_fn):
        psi, P = prep(H, psi0)
        prob = Problem(psi, P)
        rec = []

        def cb(prob, sweep, region, which, **k):
            rec.append((prob.eigenvalue, prob.last_insert.get("newdim", -1)))

        plans = [plan_fn(psi.g, nsites, **kws) for _ in range(3)]
        prob = solve(prob, plans, upd, region_callback=cb)
        return np.array(rec), prob.eigenvalue

    r, E = run(pn, lambda H_, p_: _prepare(H_, p_, nsg_ctx), EigsolveProblem, sweep_solve, updater_eigsolve,
               pn.post_order_dfs_plan)
    ro, Eo = run(on, osw._prepare, osw.EigsolveProblem, osw.sweep_solve, osw.updater_eigsolve,
                 on.post_order_dfs_plan)
    assert np.array_equal(r[:, 1], ro[:, 1])
    assert np.max(np.abs(r[:, 0] - ro[:, 0]) / np.abs(ro[:, 0])) < 1e-10
    assert abs(E - Eo) / abs(Eo) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_chain_driver_matches_general_driver(nsg_ctx, precision):
    """The chain driver (one fused region-step call per region) against the general
    driver on a J1-J2 chain with a maxdim schedule: per-region energies 1e-11 relative,
    identical bond dimensions, the same final state up to rounding."""
    from networksolvers_gb300.chain import dmrg_chain
    n = 16
    H = m.j1j2_chain(n, 0.3)
    psi0 = m.random_state(m.chain_graph(n), 8, seed=7)
    trunc = dict(cutoff=1e-10, maxdim=[16, 32, 64])
    nsg_ctx.set_precision(precision)
    try:
        Eg, rg, psig = _record_dmrg(ns.dmrg, H, psi0, nsweeps=3, nsites=2,
                                    updater_kwargs=dict(krylovdim=3, maxiter=1), inserter_kwargs=dict(trunc=trunc))
        Ec, tens, rec = dmrg_chain(H, psi0, 3, maxdim=[16, 32, 64], cutoff=1e-10, ctx=nsg_ctx)
    finally:
        nsg_ctx.set_precision("fp64")
    rc = np.array([(e, k) for (_, _, e, k) in rec])
    assert np.array_equal(rc[:, 1], rg[:, 3])
    assert np.max(np.abs(rc[:, 0] - rg[:, 2]) / np.abs(rg[:, 2])) < 1e-11
    assert abs(Ec - Eg) / abs(Eg) < 1e-11
    ref = psig.to_numpy(psi0)
    for v in ref:
        assert tens[v].shape == ref[v].shape


def test_opsum_tree_operator_dmrg_matches_oracle(nsg_ctx):
    """test_tree_dmrg.jl:18-53 with the operator compiled from the OpSum (itn.ttn(os, s),
    test_tree_dmrg.jl:28) plus a field and a next-nearest-neighbour term across the
    centre: 2-site DMRG on the three-branch tree, per-region energies 1e-10 and bond
    dimensions exact against the oracle, the energy within 1e-5 of ED for the pure
    Heisenberg OpSum."""
    from oracle import sweep as osw
    from oracle import ed
    g = m.build_tree_graph(3, 3)
    kw = dict(nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=40)))
    H = m.ttn_operator(m.heisenberg_opsum(g), g)
    E, r, _ = _record_dmrg(ns.dmrg, H, m.neel_state(g), **kw)
    Hx = ed.hamiltonian(g.vertices, ed.heisenberg_terms(g.edges))
    assert abs(E - ed.ground_energy(Hx)) < 1e-5
    os_ = m.heisenberg_opsum(g)
    os_.add(0.3, "Sz", (1, 1), "Sz", (2, 1))
    os_.add(0.2, "Sx", (3, 3))
    H2 = m.ttn_operator(os_, g)
    Eo, ro, _ = _record_dmrg(osw.dmrg, H2, m.neel_state(g), **kw)
    E2, r2, _ = _record_dmrg(ns.dmrg, H2, m.neel_state(g), **kw)
    assert np.array_equal(r2[:, 3], ro[:, 3])
    assert np.max(np.abs(r2[:, 2] - ro[:, 2]) / np.abs(ro[:, 2])) < 1e-10
    assert abs(E2 - Eo) / abs(Eo) < 1e-10
