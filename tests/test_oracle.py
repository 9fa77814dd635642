"""The oracle pinned against exact diagonalisation and the reference's own assertions
(test/dmrg/test_tree_dmrg.jl:53,67; test/tdvp/test_tree_tdvp.jl:65-77)."""
import numpy as np

import networksolvers_gb300.models as m
from oracle import sweep, ed, linalg, network


def _ed_heis(g):
    return ed.ground_energy(ed.hamiltonian(g.vertices, ed.heisenberg_terms(g.edges)))


def test_truncation_rule():
    P = np.array([0.5, 0.3, 0.1, 0.05, 0.04, 0.01])
    assert linalg.truncate_spectrum(P, cutoff=0.0)[0] == 6
    assert linalg.truncate_spectrum(P, maxdim=3)[0] == 3
    n, err = linalg.truncate_spectrum(P, cutoff=0.011)          # 0.01 < 0.011 -> drop one
    assert n == 5 and abs(err - 0.01) < 1e-15
    n, _ = linalg.truncate_spectrum(P, cutoff=0.05)              # 0.01+0.04 = 0.05 not < 0.05
    assert n == 5
    n, _ = linalg.truncate_spectrum(P, cutoff=0.0501)
    assert n == 4
    n, _ = linalg.truncate_spectrum(P, cutoff=0.9, mindim=2)
    assert n == 2
    n, _ = linalg.truncate_spectrum(np.array([1.0, 1e-20, -1e-18]), cutoff=0.0)
    assert n == 3


def test_compute_expansion():
    assert sweep.compute_expansion(10, 40) == 15
    assert sweep.compute_expansion(10, 12) == 2
    assert sweep.compute_expansion(10, 40, maxdim=12) == 2
    assert sweep.compute_expansion(10, 40, maxdim=8) == 0
    assert sweep.compute_expansion(4, 40, expansion_factor=1.1) == 5


def test_models_match_ed_hamiltonians():
    # contract each operator network into a dense matrix and compare with the ED build
    for g, H, terms, site in [
        (m.chain_graph(6), m.heisenberg_chain(6), ed.heisenberg_terms(m.chain_graph(6).edges), None),
        (m.build_tree_graph(2, 2), m.heisenberg_tree(m.build_tree_graph(2, 2)),
         ed.heisenberg_terms(m.build_tree_graph(2, 2).edges), None),
    ]:
        dense = _dense(H)
        ref = ed.hamiltonian(g.vertices, terms).toarray()
        assert np.allclose(dense, ref, atol=1e-13)
    g = m.binary_tree_graph(2)
    H = m.tfim_tree(g, h=0.7)
    terms = [(u, v, -1.0, m.PZ, m.PZ) for (u, v) in g.edges]
    ref = ed.hamiltonian(g.vertices, terms, {v: -0.7 * m.PX for v in g.vertices}).toarray()
    assert np.allclose(_dense(H), ref, atol=1e-13)
    # J1-J2
    Hj = m.j1j2_chain(6, 0.3)
    g = m.chain_graph(6)
    terms = ed.heisenberg_terms(g.edges) + ed.heisenberg_terms([(j, j + 2) for j in range(1, 5)], J=0.3)
    assert np.allclose(_dense(Hj), ed.hamiltonian(g.vertices, terms).toarray(), atol=1e-13)


def _dense(H):
    (g, T), sites = network.from_network(H)
    from oracle.tensor import contract
    full = contract(list(T.values()))
    bra = [sites[v].prime() for v in g.vertices]
    ket = [sites[v] for v in g.vertices]
    d = 2 ** len(g.vertices)
    return full.permute(bra + ket).data.reshape(d, d)


def test_chain_dmrg_vs_ed():
    H, psi0 = m.config_heisenberg_chain(10, 4, 0)
    E, psi = sweep.dmrg(H, psi0, nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=dict(cutoff=1e-12, maxdim=64)))
    assert abs(E - _ed_heis(H.graph)) < 1e-9


def test_reference_tree_dmrg():
    """test_tree_dmrg.jl:13-68: 2-site and 1-site+densitymatrix within 1e-5 of ED."""
    g = m.build_tree_graph(3, 3)
    H, p0 = m.heisenberg_tree(g), m.neel_state(g)
    Ex = _ed_heis(g)
    trunc = dict(cutoff=1e-5, maxdim=40)
    E, _ = sweep.dmrg(H, p0, nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=trunc))
    assert abs(E - Ex) < 1e-5
    E, _ = sweep.dmrg(H, p0, nsweeps=5, nsites=1, extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
                      inserter_kwargs=dict(trunc=trunc))
    assert abs(E - Ex) < 1e-5


def test_reference_tree_tdvp():
    """test_tree_tdvp.jl:24-78 on a smaller chain-plus-ancilla (N=6) to keep CPU time low:
    norms > 0.999, overlaps > 0.99, accumulated phase = E*tmax within 1e-4."""
    g = m.chain_plus_ancilla_graph(6)
    terms = {e: (m.heisenberg_bond_terms() if 0 not in e else []) for e in g.edges}
    H = m.tree_operator(g, terms)
    E, gs = sweep.dmrg(H, m.neel_state(g), nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=100)))
    Hc = H.astype(np.complex128)
    gsc = gs.copy()
    from oracle.tensor import Tensor
    for v in gsc.g.vertices:
        gsc.t[v] = Tensor(gs[v].data.astype(np.complex128), gs[v].inds)
    (g2, Ht), _ = network.from_network(Hc, site_index={v: [i for i in gs[v].inds if i.tags.startswith("Site")][0]
                                                       for v in gs.g.vertices})
    times = np.arange(0, 0.1 + 1e-9, 0.02)
    outs = []
    for nsites in (1, 2):
        P = network.ProjTTN(gsc.g, Ht)
        outs.append(sweep.applyexp(None, None, [-1j * t for t in times], nsites=nsites,
                                   inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=100)), init=(gsc.copy(), P)))
    p1, p2 = outs
    assert p1.norm() > 0.999 and p2.norm() > 0.999
    z = network.inner(p1, gsc)
    assert abs(z) > 0.99 and abs(network.inner(p1, p2)) > 0.99
    assert abs(np.arctan(z.imag / z.real) - E * 0.1) < 1e-4


def _kron_term(n, factors):
    mats = [np.eye(2) for _ in range(n)]
    for site, mat in factors:
        mats[site - 1] = mats[site - 1] @ mat
    out = np.array([[1.0]])
    for mt in mats:
        out = np.kron(out, mt)
    return out


def test_opsum_chain_mpo_matches_dense_sums():
    """OpSum -> chain MPO (finite-state construction) against the dense sum of Kronecker
    products: the Heisenberg chain (same operator as the hand-built MPO, bond dim 5) and
    a random mix of fields, long-range two-site and three-site terms."""
    n = 6
    os_ = m.OpSum()
    for j in range(1, n):
        os_.add(1.0, "Sz", j, "Sz", j + 1)
        os_.add(0.5, "S+", j, "S-", j + 1)
        os_.add(0.5, "S-", j, "S+", j + 1)
    H = m.chain_mpo(os_, n)
    assert max(t.shape[0] for t in H.tensors.values()) == 5
    assert np.allclose(_dense(H), _dense(m.heisenberg_chain(n)), atol=1e-13)
    rng = np.random.default_rng(4)
    n = 5
    os_ = m.OpSum()
    ref = np.zeros((2 ** n, 2 ** n))
    names = ["Sz", "S+", "S-", "Sx", "X", "Z", "N"]
    for _ in range(12):
        k = int(rng.integers(1, 4))
        sites = sorted(rng.choice(np.arange(1, n + 1), size=k, replace=False).tolist())
        ops = [names[int(rng.integers(len(names)))] for _ in sites]
        c = float(rng.standard_normal())
        args = []
        for o, s_ in zip(ops, sites):
            args += [o, s_]
        os_.add(c, *args)
        ref += c * _kron_term(n, [(s_, m.SITE_OPS[o]) for o, s_ in zip(ops, sites)])
    os_.add(0.3, "S+", 2, "S-", 2, "Sz", 4)  # two operators on one site multiply in order
    ref += 0.3 * _kron_term(n, [(2, m.SP @ m.SM), (4, m.SZ)])
    assert np.allclose(_dense(m.chain_mpo(os_, n)), ref, atol=1e-12)


def _dense_seq(H):
    """Dense matrix of an operator network, contracted vertex by vertex in vertex order
    (an exhaustive contraction-order search is too slow for ten tensors)."""
    (g, T), sites = network.from_network(H)
    acc = None
    for v in g.vertices:
        acc = T[v] if acc is None else acc * T[v]
    bra = [sites[v].prime() for v in g.vertices]
    ket = [sites[v] for v in g.vertices]
    d = 2 ** len(g.vertices)
    return acc.permute(bra + ket).data.reshape(d, d)


def _kron_tree(vertices, factors):
    pos = {v: k for k, v in enumerate(vertices)}
    mats = [np.eye(2, dtype=complex) for _ in vertices]
    for site, mat in factors:
        mats[pos[site]] = mats[pos[site]] @ mat
    out = np.array([[1.0 + 0j]])
    for mt in mats:
        out = np.kron(out, mt)
    return out


def test_opsum_ttn_operator_matches_dense_sums():
    """OpSum -> tree operator (finite-state construction on a rooted tree) against the
    dense sum of Kronecker products: the Heisenberg OpSum of test_tree_dmrg.jl:21-27 on
    the 10-site three-branch tree (equal to the hand-built tree operator, link dimension
    5, for every choice of root), and random 1-, 2- and 3-site terms, including two
    operators on one vertex and a complex coefficient, on a 7-site binary tree."""
    g = m.build_tree_graph(3, 3)
    ref = _dense_seq(m.heisenberg_tree(g))
    for root in (None, (0, 0), (2, 3)):
        H = m.ttn_operator(m.heisenberg_opsum(g), g, root=root)
        assert max(max(t.shape) for t in H.tensors.values()) == 5
        assert np.allclose(_dense_seq(H), ref, atol=1e-13)
    g = m.binary_tree_graph(2)
    rng = np.random.default_rng(7)
    os_ = m.OpSum()
    dense = np.zeros((2 ** 7, 2 ** 7), dtype=complex)
    names = ["Sz", "S+", "S-", "Sx", "Sy", "X", "Z", "N"]
    for _ in range(14):
        k = int(rng.integers(1, 4))
        sites = [g.vertices[i] for i in rng.choice(len(g.vertices), size=k, replace=False)]
        ops = [names[int(rng.integers(len(names)))] for _ in sites]
        c = float(rng.standard_normal())
        args = []
        for o, s_ in zip(ops, sites):
            args += [o, s_]
        os_.add(c, *args)
        dense += c * _kron_tree(g.vertices, [(s_, m.SITE_OPS[o]) for o, s_ in zip(ops, sites)])
    os_.add(0.25 - 0.5j, "S+", 3, "S-", 3, "Z", 6)
    dense += (0.25 - 0.5j) * _kron_tree(g.vertices, [(3, m.SP @ m.SM), (6, m.PZ)])
    for root in (None, 0, 4):
        H = m.ttn_operator(os_, g, root=root)
        assert np.allclose(_dense_seq(H), dense, atol=1e-12)
    # on a chain it is the chain MPO's operator
    n = 5
    osc = m.OpSum()
    for j in range(1, n):
        osc.add(0.7, "Sz", j, "Sz", j + 1)
        osc.add(0.3, "X", j)
    assert np.allclose(_dense_seq(m.ttn_operator(osc, m.chain_graph(n))), _dense_seq(m.chain_mpo(osc, n)), atol=1e-13)


def test_opsum_ttn_tree_dmrg_vs_ed():
    """test_tree_dmrg.jl:18-53 with the operator built from the OpSum (itn.ttn(os, s),
    test_tree_dmrg.jl:28): 2-site DMRG on the three-branch tree within 1e-5 of ED."""
    g = m.build_tree_graph(3, 3)
    H = m.ttn_operator(m.heisenberg_opsum(g), g)
    E, _ = sweep.dmrg(H, m.neel_state(g), nsweeps=5, nsites=2,
                      inserter_kwargs=dict(trunc=dict(cutoff=1e-5, maxdim=40)))
    assert abs(E - _ed_heis(g)) < 1e-5
