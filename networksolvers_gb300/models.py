"""Input formats for the sweep: graphs, tree/chain operators and initial states.

Everything here is host-side numpy and builds the *inputs* that the reference
obtains from `itn.siteinds`, `itn.mpo(os, s)` / `itn.ttn(os, s)`,
`itn.random_mps(s; link_space)` and `itn.ttn(state, s)`
(test/dmrg/test_tree_dmrg.jl:18-35, examples/dmrg.jl:264-278).

Plain-data exchange format (consumed by the device path and by the CPU oracle):

* ``Graph``: vertices in insertion order, edges as added.  ``edges_sorted``
  follows Graphs.jl's SimpleGraph edge order (by insertion position), which is
  what `compute_adjacencies` in region_plans/euler_tour.jl:4-11 iterates.
* A network is ``(tensors, legs)``: ``tensors[v]`` is a numpy array whose axes
  are named by ``legs[v]``.  Leg names: ``('s', v)`` site (ket), ``('sp', v)``
  primed site (bra side of an operator), ``('l', e)`` state link on edge ``e``,
  ``('w', e)`` operator link on edge ``e``.  The leg order follows
  permute_indices.jl:4-18: first link, then site(s), then the other links.
  The device receives each array in column-major order with these axes, which
  is the memory layout of the corresponding ITensor.

Operator tensors hold ``W[..., s', s] = <s'|O|s>``.  Site basis for S=1/2 is
(Up, Dn), as ITensors' "S=1/2" site type.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import numpy as np

# ----------------------------------------------------------------------------
# Graphs
# ----------------------------------------------------------------------------


@dataclass
class Graph:
    vertices: list
    edges: list  # (u, v) as added

    def __post_init__(self):
        self.pos = {v: i for i, v in enumerate(self.vertices)}
        self.edges = [self.edge_key(u, v) for (u, v) in self.edges]

    def edge_key(self, u, v):
        """Canonical undirected edge key: endpoints ordered by insertion position."""
        return (u, v) if self.pos[u] < self.pos[v] else (v, u)

    @property
    def edges_sorted(self):
        return sorted(self.edges, key=lambda e: (self.pos[e[0]], self.pos[e[1]]))

    def neighbors(self, v):
        """Neighbours in ascending insertion position (Graphs.jl `neighbors` order)."""
        out = []
        for (a, b) in self.edges:
            if a == v:
                out.append(b)
            elif b == v:
                out.append(a)
        return sorted(out, key=lambda x: self.pos[x])

    def link_neighbors(self, v):
        """Neighbours in the order the vertex's link legs are stored (edge creation order)."""
        out = []
        for (a, b) in self.edges:
            if a == v:
                out.append(b)
            elif b == v:
                out.append(a)
        return out

    def is_leaf(self, v):
        return len(self.neighbors(v)) == 1

    def leaf_vertices(self):
        return [v for v in self.vertices if self.is_leaf(v)]


def chain_graph(n):
    return Graph(list(range(1, n + 1)), [(j, j + 1) for j in range(1, n)])


def binary_tree_graph(depth):
    """Complete binary tree with levels 0..depth (2^(depth+1)-1 vertices, BFS numbering)."""
    nv = 2 ** (depth + 1) - 1
    verts = list(range(nv))
    edges = [((c - 1) // 2, c) for c in range(1, nv)]
    return Graph(verts, edges)


def build_tree_graph(nbranch=3, nbranch_sites=3):
    """Star of `nbranch` chains around (0,0) — test/utilities/tree_graphs.jl:10-23."""
    verts = [(0, 0)] + [(b, s) for b in range(1, nbranch + 1) for s in range(1, nbranch_sites + 1)]
    edges = []
    for b in range(1, nbranch + 1):
        edges.append(((0, 0), (b, 1)))
        for s in range(2, nbranch_sites + 1):
            edges.append(((b, s - 1), (b, s)))
    return Graph(verts, edges)


def chain_plus_ancilla_graph(nchain):
    """Chain 1..n plus vertex 0 attached to n÷2 — test/tdvp/test_tree_tdvp.jl:10-22."""
    verts = list(range(1, nchain + 1)) + [0]
    edges = [(j, j + 1) for j in range(1, nchain)] + [(0, nchain // 2)]
    return Graph(verts, edges)


# ----------------------------------------------------------------------------
# Local operators
# ----------------------------------------------------------------------------

SZ = np.array([[0.5, 0.0], [0.0, -0.5]])
SP = np.array([[0.0, 1.0], [0.0, 0.0]])
SM = np.array([[0.0, 0.0], [1.0, 0.0]])
PZ = np.array([[1.0, 0.0], [0.0, -1.0]])
PX = np.array([[0.0, 1.0], [1.0, 0.0]])
ID2 = np.eye(2)


def heisenberg_bond_terms(J=1.0, delta=1.0):
    """(coef, op_i, op_j) for J*(Δ Sz Sz + ½ S+S- + ½ S-S+)."""
    return [(J * delta, SZ, SZ), (0.5 * J, SP, SM), (0.5 * J, SM, SP)]


def ising_bond_terms(J=1.0):
    """-J Z Z."""
    return [(-J, PZ, PZ)]


# ----------------------------------------------------------------------------
# Operator networks
# ----------------------------------------------------------------------------


@dataclass
class Network:
    graph: Graph
    tensors: dict
    legs: dict
    dtype: type = np.float64
    meta: dict = field(default_factory=dict)

    def site_dim(self, v):
        t, lg = self.tensors[v], self.legs[v]
        return t.shape[lg.index(('s', v))]

    def link_dim(self, e):
        u = e[0]
        t, lg = self.tensors[u], self.legs[u]
        key = ('l', e) if ('l', e) in lg else ('w', e)
        return t.shape[lg.index(key)]

    def astype(self, dtype):
        return Network(self.graph, {v: t.astype(dtype) for v, t in self.tensors.items()},
                       dict(self.legs), dtype, dict(self.meta))


def _permuted_legs(graph, v, link_kind, site_legs):
    """Leg order of permute_indices.jl:4-18: [first link, site legs..., other links]."""
    links = [(link_kind, graph.edge_key(v, u)) for u in graph.link_neighbors(v)]
    if not links:
        return list(site_legs)
    return [links[0]] + list(site_legs) + links[1:]


def tree_operator(graph, bond_terms, site_terms=None, root=None):
    """TTN operator for H = Σ_edges Σ_t c_t A_t(i) B_t(j) + Σ_v h_v.

    Built as a finite-state automaton on a rooted tree.  The link from a vertex to its
    parent carries one of: 0 = identity, 1..T = term t pending (its operator sits at the
    child, the partner sits at the parent), T+1 = complete.  Link dimension = T + 2
    (5 for Heisenberg, 3 for transverse-field Ising).  `bond_terms` is either a list of
    (coef, A, B) applied to every edge, or a dict edge -> list.
    `site_terms`: dict v -> d×d matrix (or None).
    """
    if root is None:
        root = graph.vertices[-1]
    site_terms = site_terms or {}
    d = 2
    parent = {root: None}
    order = [root]
    k = 0
    while k < len(order):
        v = order[k]
        for u in graph.neighbors(v):
            if u not in parent:
                parent[u] = v
                order.append(u)
        k += 1

    def terms_on(e):
        if isinstance(bond_terms, dict):
            return bond_terms.get(e, [])
        return bond_terms

    tensors, legs = {}, {}
    for v in graph.vertices:
        p = parent[v]
        children = [u for u in graph.neighbors(v) if parent.get(u) == v]
        # dims
        def wdim(e):
            return len(terms_on(e)) + 2
        link_order = [graph.edge_key(v, u) for u in graph.link_neighbors(v)]
        dims = {e: wdim(e) for e in link_order}
        # build in an internal axis order: [parent?, children..., s', s]
        axes_e = ([graph.edge_key(v, p)] if p is not None else []) + [graph.edge_key(v, c) for c in children]
        shape = [dims[e] for e in axes_e] + [d, d]
        W = np.zeros(shape)
        nch = len(children)

        def put(pstate, cstates, op):
            idx = ([pstate] if p is not None else []) + list(cstates)
            W[tuple(idx)] += op

        zero_c = [0] * nch
        ep = graph.edge_key(v, p) if p is not None else None
        complete_p = (len(terms_on(ep)) + 1) if p is not None else None
        if p is not None:
            put(0, zero_c, ID2)
            for t, (c, A, B) in enumerate(terms_on(ep)):
                # operator at the child end of edge (v, p); v is the child
                opv = A if ep[0] == v else B
                put(1 + t, zero_c, opv)
        # "complete" slice (the only slice for the root)
        cp = complete_p

        def put_complete(cstates, op):
            if p is None:
                W[tuple(cstates)] += op
            else:
                put(cp, cstates, op)

        if v in site_terms and site_terms[v] is not None:
            put_complete(zero_c, site_terms[v])
        for i, ch in enumerate(children):
            ec = graph.edge_key(v, ch)
            tc = terms_on(ec)
            cs = list(zero_c)
            cs[i] = len(tc) + 1
            put_complete(cs, ID2)
            for t, (c, A, B) in enumerate(tc):
                cs = list(zero_c)
                cs[i] = 1 + t
                # v is the parent end of edge ec
                opv = A if ec[0] == v else B
                put_complete(cs, c * opv)
        # permute to the stored leg order
        internal = [('w', e) for e in axes_e] + [('sp', v), ('s', v)]
        target = _permuted_legs(graph, v, 'w', [('sp', v), ('s', v)])
        perm = [internal.index(l) for l in target]
        tensors[v] = np.ascontiguousarray(W.transpose(perm))
        legs[v] = target
    return Network(graph, tensors, legs, np.float64, {"kind": "operator"})


def chain_operator(n, J1=1.0, J2=0.0, delta=1.0, h=None):
    """Chain MPO for Σ J1 (Δ SzSz + ½S+S- + ½S-S+)_{i,i+1} + J2 (same)_{i,i+2}.

    States (left to right): start, 3 pending-at-distance-1, [3 pending-at-distance-2],
    done.  Link dimension 5 for J2 == 0 (Heisenberg/XXZ), 8 otherwise (J1-J2).
    `h`: optional on-site field (d×d matrix added at every site).
    """
    g = chain_graph(n)
    ops = [(delta, SZ, SZ), (0.5, SP, SM), (0.5, SM, SP)]
    nt = len(ops)
    use2 = J2 != 0.0
    w = 2 + nt + (nt if use2 else 0)
    START, DONE = 0, w - 1
    P1 = lambda t: 1 + t
    P2 = lambda t: 1 + nt + t
    Wb = np.zeros((w, w, 2, 2))  # [left, right, s', s]
    Wb[START, START] = ID2
    Wb[DONE, DONE] = ID2
    if h is not None:
        Wb[START, DONE] += h
    for t, (c, A, B) in enumerate(ops):
        Wb[START, P1(t)] += A
        Wb[P1(t), DONE] += J1 * c * B
        if use2:
            Wb[P1(t), P2(t)] += ID2
            Wb[P2(t), DONE] += J2 * c * B
    tensors, legs = {}, {}
    for j in g.vertices:
        if n == 1:
            T = Wb[START, DONE]
            tensors[j] = T.copy()
            legs[j] = [('sp', j), ('s', j)]
            continue
        el = g.edge_key(j - 1, j) if j > 1 else None
        er = g.edge_key(j, j + 1) if j < n else None
        if j == 1:
            T = Wb[START]                       # [right, s', s]
            tensors[j] = np.ascontiguousarray(T.transpose(0, 1, 2))
            legs[j] = [('w', er), ('sp', j), ('s', j)]
        elif j == n:
            T = Wb[:, DONE]                     # [left, s', s]
            tensors[j] = np.ascontiguousarray(T)
            legs[j] = [('w', el), ('sp', j), ('s', j)]
        else:
            T = Wb.transpose(0, 2, 3, 1)        # [left, s', s, right]
            tensors[j] = np.ascontiguousarray(T)
            legs[j] = [('w', el), ('sp', j), ('s', j), ('w', er)]
    return Network(g, tensors, legs, np.float64, {"kind": "operator", "w": w})


# ----------------------------------------------------------------------------
# OpSum -> chain MPO (the input format of the reference's tests and examples: itn.mpo /
# itn.ttn of an OpSum, e.g. test_tree_dmrg.jl:28)
# ----------------------------------------------------------------------------

SITE_OPS = {"Sz": SZ, "S+": SP, "S-": SM, "Sx": 0.5 * PX, "Id": ID2, "X": PX, "Z": PZ,
            "Sy": np.array([[0.0, -0.5j], [0.5j, 0.0]]), "Y": np.array([[0.0, -1.0j], [1.0j, 0.0]]),
            "N": np.array([[0.0, 0.0], [0.0, 1.0]])}


class OpSum:
    """A sum of products of on-site operators, written as in ITensors:
    `os.add(coef, "Sz", i, "Sz", j)` or `os += (coef, "S+", i, "S-", j)`.  Operators are
    names of SITE_OPS (S=1/2 basis order Up, Dn) or d x d arrays; sites are 1-based
    integers on a chain and vertex names (any hashable) on a tree."""

    def __init__(self):
        self.terms = []

    def add(self, coef, *ops):
        if len(ops) % 2 or not ops:
            raise ValueError("OpSum.add(coef, op1, site1, op2, site2, ...)")
        factors = []
        for k in range(0, len(ops), 2):
            op, site = ops[k], ops[k + 1]
            if isinstance(site, (int, np.integer)):
                site = int(site)
            mat = SITE_OPS[op] if isinstance(op, str) else np.asarray(op)
            factors.append((site, mat))
        self.terms.append((coef, factors))
        return self

    def __iadd__(self, term):
        return self.add(*term)


def chain_mpo(opsum, n, d=2):
    """Exact MPO of an OpSum on a chain of n sites by the finite-state construction: on
    the bond (j, j+1) the automaton is in START (no operator placed), DONE (all placed) or
    in the private state of one term whose first site is <= j and last site > j, so the
    bond dimension is 2 + the number of terms spanning it (5 for the Heisenberg chain).
    Operators of one term on the same site multiply in the order given."""
    g = chain_graph(n)
    cplx = any(np.iscomplexobj(m) or np.iscomplexobj(c) for c, fs in opsum.terms for _, m in fs)
    dt = np.complex128 if cplx else np.float64
    START, DONE = 0, 1
    terms = []
    for c, fs in opsum.terms:
        per = {}
        for site, mat in fs:
            if not 1 <= site <= n:
                raise ValueError(f"OpSum site {site} outside 1..{n}")
            per[site] = per[site] @ mat if site in per else np.asarray(mat, dtype=dt)
        sites = sorted(per)
        terms.append((c, per, sites[0], sites[-1]))
    # bond states: bond b between sites b and b+1 (b = 1..n-1)
    state = {}
    bdim = {}
    for b in range(1, n):
        k = 2
        for t, (_, _, f, l) in enumerate(terms):
            if f <= b < l:
                state[(t, b)] = k
                k += 1
        bdim[b] = k
    ident = np.eye(d, dtype=dt)
    tensors, legs = {}, {}
    for j in range(1, n + 1):
        wl = bdim.get(j - 1, 1)
        wr = bdim.get(j, 1)
        W = np.zeros((wl, d, d, wr), dtype=dt)   # [left, s', s, right]
        lstart = 0 if j > 1 else 0
        rdone = 1 if j < n else 0
        if j > 1:
            W[DONE, :, :, rdone] += ident
        if j < n:
            W[lstart, :, :, START] += ident
        for t, (c, per, f, l) in enumerate(terms):
            op = per.get(j, ident)
            if f == l == j:
                W[lstart, :, :, rdone] += c * op
            elif f == j:
                W[lstart, :, :, state[(t, j)]] += c * op
            elif f < j < l:
                W[state[(t, j - 1)], :, :, state[(t, j)]] += op
            elif j == l and f < j:
                W[state[(t, j - 1)], :, :, rdone] += op
        el = g.edge_key(j - 1, j) if j > 1 else None
        er = g.edge_key(j, j + 1) if j < n else None
        if n == 1:
            tensors[j] = W[0, :, :, 0].copy()
            legs[j] = [('sp', j), ('s', j)]
        elif j == 1:
            tensors[j] = np.ascontiguousarray(W[0].transpose(2, 0, 1))   # [right, s', s]
            legs[j] = [('w', er), ('sp', j), ('s', j)]
        elif j == n:
            tensors[j] = np.ascontiguousarray(W[:, :, :, 0])            # [left, s', s]
            legs[j] = [('w', el), ('sp', j), ('s', j)]
        else:
            tensors[j] = np.ascontiguousarray(W)
            legs[j] = [('w', el), ('sp', j), ('s', j), ('w', er)]
    return Network(g, tensors, legs, dt, {"kind": "operator", "w": max(bdim.values()) if bdim else 1})


def ttn_operator(opsum, graph, root=None, d=2):
    """Exact tree operator (TTN) of an OpSum on a tree graph: the finite-state
    construction of `chain_mpo` on a rooted tree (the input format `itn.ttn(os, sites)` of
    the reference's tests, e.g. test_tree_dmrg.jl:28).

    Rooted at `root` (default: the last vertex), every edge (child c, parent p) carries
    the automaton state of the subtree below it: IDENT (identity everywhere below),
    DONE (exactly one term completed below) or, for each term whose support lies partly
    below and partly above the edge, that term's private state.  Link dimension = 2 +
    the number of terms crossing the edge (5 on every edge of a nearest-neighbour
    Heisenberg tree).  A vertex tensor sends: all children IDENT -> IDENT (identity);
    one child DONE, the others IDENT -> DONE (identity); and, for each term with support
    in its subtree that does not lie below a single child, the children holding part of
    the term in that term's state, the others IDENT, to the term's state (the term
    continues above) or to DONE (the vertex is the term's topmost vertex, where the
    coefficient is applied), with the term's operator at the vertex (identity when the
    vertex only joins parts of the support).  The root keeps only the DONE output.
    Operators of one term on the same vertex multiply in the order given."""
    verts = list(graph.vertices)
    if root is None:
        root = verts[-1]
    parent = {root: None}
    order = [root]
    k = 0
    while k < len(order):
        v = order[k]
        for u in graph.neighbors(v):
            if u not in parent:
                parent[u] = v
                order.append(u)
        k += 1
    if len(order) != len(verts):
        raise ValueError("ttn_operator: the graph is not a connected tree")
    children = {v: [u for u in graph.neighbors(v) if parent.get(u) == v] for v in verts}
    below = {}
    for v in reversed(order):  # leaves first
        sset = {v}
        for c_ in children[v]:
            sset |= below[c_]
        below[v] = sset
    cplx = any(np.iscomplexobj(m_) or np.iscomplexobj(c_) for c_, fs in opsum.terms for _, m_ in fs)
    dt = np.complex128 if cplx else np.float64
    ident = np.eye(d, dtype=dt)
    terms = []
    for c_, fs in opsum.terms:
        per = {}
        for site, mat in fs:
            if site not in parent:
                raise ValueError(f"OpSum site {site!r} is not a vertex of the graph")
            per[site] = per[site] @ mat if site in per else np.asarray(mat, dtype=dt)
        terms.append((c_, per, set(per)))
    IDENT, DONE = 0, 1
    # private states: edge (c -> parent) for every term crossing it
    state, wdim = {}, {}
    for v in verts:
        if parent[v] is None:
            continue
        kk = 2
        for t, (_, _, sup) in enumerate(terms):
            if sup & below[v] and not sup <= below[v]:
                state[(t, v)] = kk
                kk += 1
        wdim[v] = kk
    tensors, legs = {}, {}
    for v in verts:
        p, ch = parent[v], children[v]
        shape = ([wdim[v]] if p is not None else []) + [wdim[c_] for c_ in ch] + [d, d]
        W = np.zeros(shape, dtype=dt)

        def put(pstate, cstates, op):
            if p is None and pstate != DONE:
                return
            idx = ([pstate] if p is not None else []) + list(cstates)
            W[tuple(idx)] += op

        zero = [IDENT] * len(ch)
        put(IDENT, zero, ident)
        for i in range(len(ch)):
            cs = list(zero)
            cs[i] = DONE
            put(DONE, cs, ident)
        for t, (coef, per, sup) in enumerate(terms):
            if not sup & below[v]:
                continue
            if any(sup <= below[c_] for c_ in ch):
                continue  # the term completes inside one child's subtree
            cs = [state[(t, c_)] if sup & below[c_] else IDENT for c_ in ch]
            op = per.get(v, ident)
            if sup <= below[v]:
                put(DONE, cs, coef * op)
            else:
                put(state[(t, v)], cs, op)
        # stored leg order [first link, s', s, other links] (permute_indices.jl:4-18)
        internal = ([('w', graph.edge_key(v, p))] if p is not None else []) + \
                   [('w', graph.edge_key(v, c_)) for c_ in ch] + [('sp', v), ('s', v)]
        target = _permuted_legs(graph, v, 'w', [('sp', v), ('s', v)])
        perm = [internal.index(l_) for l_ in target]
        tensors[v] = np.ascontiguousarray(W.transpose(perm))
        legs[v] = target
    return Network(graph, tensors, legs, dt, {"kind": "operator", "w": max(wdim.values()) if wdim else 1})


def heisenberg_opsum(graph, J=1.0, delta=1.0):
    """The OpSum of test_tree_dmrg.jl:21-27: Σ_edges J (Δ Sz Sz + ½ S+ S- + ½ S- S+)."""
    os_ = OpSum()
    for (u, v) in graph.edges:
        os_.add(J * delta, "Sz", u, "Sz", v)
        os_.add(0.5 * J, "S+", u, "S-", v)
        os_.add(0.5 * J, "S-", u, "S+", v)
    return os_


def heisenberg_chain(n, J=1.0):
    return chain_operator(n, J1=J, J2=0.0, delta=1.0)


def xxz_chain(n, delta, J=1.0):
    return chain_operator(n, J1=J, J2=0.0, delta=delta)


def j1j2_chain(n, J2, J1=1.0):
    return chain_operator(n, J1=J1, J2=J2, delta=1.0)


def tfim_tree(graph, h=1.0, J=1.0, root=None):
    """H = -J Σ_<ij> Z_i Z_j - h Σ_i X_i on a tree (Pauli matrices)."""
    site = {v: -h * PX for v in graph.vertices}
    return tree_operator(graph, ising_bond_terms(J), site, root=root)


def heisenberg_tree(graph, J=1.0):
    return tree_operator(graph, heisenberg_bond_terms(J))


# ----------------------------------------------------------------------------
# States
# ----------------------------------------------------------------------------


def random_state(graph, link_space, seed=0, dtype=np.float64, d=2):
    """Random tree tensor network with every link of dimension `link_space`.

    Own seeded generator (Julia's RNG stream cannot be reproduced): numpy PCG64 with
    `seed`, standard-normal entries drawn vertex by vertex in vertex order, each tensor
    filled in its stored (row-major numpy) axis order; for complex dtypes the real part
    and then the imaginary part of each tensor are drawn before the next vertex.
    The orthogonality region is all vertices (not orthogonalised), so the first
    extract step QR-walks every tensor toward the first region, as for any
    non-orthogonal input state.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    tensors, legs = {}, {}
    for v in graph.vertices:
        lg = _permuted_legs(graph, v, 'l', [('s', v)])
        shape = [d if l[0] == 's' else link_space for l in lg]
        if np.issubdtype(dtype, np.complexfloating):
            t = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        else:
            t = rng.standard_normal(shape)
        tensors[v] = t.astype(dtype)
        legs[v] = lg
    return Network(graph, tensors, legs, dtype, {"kind": "state", "ortho_region": list(graph.vertices)})


def product_state(graph, local_states, dtype=np.float64, d=2):
    """Product state with link dimension 1.  `local_states[v]` is a length-d vector
    or the string "Up"/"Dn" (S=1/2 basis order (Up, Dn))."""
    tensors, legs = {}, {}
    for v in graph.vertices:
        s = local_states[v]
        if isinstance(s, str):
            vec = np.zeros(d)
            vec[{"Up": 0, "Dn": 1}[s]] = 1.0
        else:
            vec = np.asarray(s)
        lg = _permuted_legs(graph, v, 'l', [('s', v)])
        shape = [d if l[0] == 's' else 1 for l in lg]
        t = np.zeros(shape, dtype=dtype)
        idx = [slice(None) if l[0] == 's' else 0 for l in lg]
        t[tuple(idx)] = vec
        tensors[v] = t
        legs[v] = lg
    return Network(graph, tensors, legs, dtype, {"kind": "state", "ortho_region": list(graph.vertices)})


def neel_state(graph, dtype=np.float64):
    """Up on even positions (1-based), Dn on odd — test/dmrg/test_tree_dmrg.jl:31-34."""
    st = {v: ("Up" if (j + 1) % 2 == 0 else "Dn") for j, v in enumerate(graph.vertices)}
    return product_state(graph, st, dtype)


def all_up_state(graph, dtype=np.complex128):
    return product_state(graph, {v: "Up" for v in graph.vertices}, dtype)


# ----------------------------------------------------------------------------
# Workload configurations (synthetic inputs with the configs' shapes)
# ----------------------------------------------------------------------------


def config_heisenberg_chain(n=20, chi0=10, seed=0):
    """Heisenberg chain, random MPS at bond dim chi0 (configs: N=20/χ0=10/seed 0 and
    N=100/χ0=32/seed 1)."""
    return heisenberg_chain(n), random_state(chain_graph(n), chi0, seed)


def config_tfim_tree(depth=5, h=1.0):
    g = binary_tree_graph(depth)
    return tfim_tree(g, h=h).astype(np.complex128), all_up_state(g)


def config_j1j2_batch(k):
    """Chain k of the batched workload: N~U[16,64], J2~U[0,0.5], maxdim~U{32,64,128}, χ0=8."""
    rng = np.random.Generator(np.random.PCG64(1000 + k))
    n = int(rng.integers(16, 65))
    j2 = float(rng.uniform(0.0, 0.5))
    maxdim = int(rng.choice([32, 64, 128]))
    return dict(n=n, J2=j2, maxdim=maxdim, seed=k,
                H=j1j2_chain(n, j2), psi0=random_state(chain_graph(n), 8, seed=k))
