"""Tree tensor networks, the projected operator and region plans (test infrastructure).

* `TTN` — vertex tensors with ITensor-style indices, an orthogonality region and a
  modification stamp per vertex (used to tell which cached environments are stale).
* `orthogonalize` — ITensorNetworks `orthogonalize(ψ, region)` as used at
  extracter.jl:6: QR along `edge_sequence_between_regions(ortho_region, region)`:
  the Steiner tree of both regions, post-order DFS edges rooted at first(region),
  without edges inside the new region.
* `ProjTTN` — ITensorNetworks `ProjTTN`: one environment per directed edge u→v
  (contraction of bra, operator and ket over the subtree on u's side), with indices
  (link', operator link, link).  An environment is recomputed whenever a tensor on
  its side changed since it was cached (`position`, extracter.jl:14).
* `optimal_map` — operator_map.jl:3-10.
* Region plans — euler_tour.jl:4-48, euler_plans.jl:4-13, dfs_plans.jl:5-22,
  tdvp_region_plans.jl:1-44.  `default_root_vertex` (NamedGraphs, un-vendored) is
  restated as the first leaf vertex in vertex order.
"""
from __future__ import annotations

import itertools

import numpy as np

from .tensor import Index, Tensor, contract, uniqueinds, commonind
from . import linalg

_stamp = itertools.count(1)


# ----------------------------------------------------------------------------
# Graph helpers (restated Graphs.jl / NamedGraphs behaviour)
# ----------------------------------------------------------------------------


class G:
    def __init__(self, vertices, edges):
        self.vertices = list(vertices)
        self.pos = {v: i for i, v in enumerate(self.vertices)}
        self.edges = [self.key(u, v) for (u, v) in edges]
        self.adjn = {v: [] for v in self.vertices}
        for (u, v) in self.edges:
            self.adjn[u].append(v)
            self.adjn[v].append(u)
        for v in self.vertices:
            self.adjn[v].sort(key=lambda x: self.pos[x])

    def key(self, u, v):
        return (u, v) if self.pos[u] < self.pos[v] else (v, u)

    def neighbors(self, v):
        return self.adjn[v]

    def edges_sorted(self):
        return sorted(self.edges, key=lambda e: (self.pos[e[0]], self.pos[e[1]]))

    def leaves(self):
        return [v for v in self.vertices if len(self.adjn[v]) == 1]

    def default_root_vertex(self):
        lv = self.leaves()
        return lv[0] if lv else self.vertices[0]

    def side(self, u, v):
        """Vertices on u's side of edge (u, v)."""
        seen = {u}
        stack = [u]
        while stack:
            x = stack.pop()
            for y in self.adjn[x]:
                if y not in seen and not (x == u and y == v):
                    seen.add(y)
                    stack.append(y)
        return seen


def post_order_dfs_vertices(g: G, root, allowed=None):
    out = []
    seen = {root}

    def visit(v):
        for u in g.neighbors(v):
            if (allowed is None or u in allowed) and u not in seen:
                seen.add(u)
                visit(u)
        out.append(v)

    visit(root)
    return out


def post_order_dfs_edges(g: G, root, allowed=None):
    """Edges (child → parent) in post order."""
    parent = {root: None}
    order = []
    seen = {root}

    def visit(v):
        for u in g.neighbors(v):
            if (allowed is None or u in allowed) and u not in seen:
                seen.add(u)
                parent[u] = v
                visit(u)
        order.append(v)

    visit(root)
    return [(v, parent[v]) for v in order if parent[v] is not None]


def steiner_tree(g: G, terminals):
    """Minimal subtree containing `terminals` (prune non-terminal leaves)."""
    keep = set(g.vertices)
    terms = set(terminals)
    changed = True
    while changed:
        changed = False
        for v in list(keep):
            if v in terms:
                continue
            deg = sum(1 for u in g.neighbors(v) if u in keep)
            if deg <= 1:
                keep.discard(v)
                changed = True
    return keep


def edge_sequence_between_regions(g: G, region1, region2):
    if set(region1) == set(region2):
        return []
    st = steiner_tree(g, list(region1) + list(region2))
    path = post_order_dfs_edges(g, region2[0], allowed=st)
    return [(s, d) for (s, d) in path if not (s in region2 and d in region2)]


# ----------------------------------------------------------------------------
# Region plans
# ----------------------------------------------------------------------------


def euler_tour_edges(g: G, start):
    adj = {v: [] for v in g.vertices}
    for (s, d) in g.edges_sorted():
        adj[s].append(d)
        adj[d].append(s)
    visited = set()
    tour = []
    stack = [start]
    while stack:
        u = stack[-1]
        pushed = False
        for v in adj[u]:
            if (u, v) not in visited:
                visited.add((u, v))
                visited.add((v, u))
                tour.append((u, v))
                stack.append(v)
                pushed = True
                break
        if not pushed:
            stack.pop()
            if stack:
                tour.append((u, stack[-1]))
    return tour


def euler_tour_vertices(g: G, start):
    edges = euler_tour_edges(g, start)
    if not edges:
        return []
    return [edges[0][0]] + [e[1] for e in edges]


def euler_sweep(g: G, nsites, root_vertex=None, **sweep_kwargs):
    root = g.default_root_vertex() if root_vertex is None else root_vertex
    if nsites == 1:
        return [([v], dict(sweep_kwargs)) for v in euler_tour_vertices(g, root)]
    return [([s, d], dict(sweep_kwargs)) for (s, d) in euler_tour_edges(g, root)]


def post_order_dfs_plan(g: G, nsites, root_vertex=None, **sweep_kwargs):
    root = g.default_root_vertex() if root_vertex is None else root_vertex
    if nsites == 1:
        return [([v], dict(sweep_kwargs)) for v in post_order_dfs_vertices(g, root)]
    return [([s, d], dict(sweep_kwargs)) for (s, d) in post_order_dfs_edges(g, root)]


def tdvp_sub_time_steps(order):
    if order == 1:
        return [1.0]
    if order == 2:
        return [0.5, 0.5]
    if order == 4:
        s = (2 - 2 ** (1 / 3)) ** (-1)
        return [s / 2, s / 2, 0.5 - s, 0.5 - s, s / 2, s / 2]
    raise ValueError(f"TDVP order of {order} not supported")


def first_order_sweep(g: G, time_step, forward, updater_kwargs, nsites, **kws):
    basic = post_order_dfs_plan(g, nsites, **kws)
    upd = dict(nsites=nsites, time_step=time_step, **updater_kwargs)
    sweep = []
    for j, (region, rkws) in enumerate(basic):
        sweep.append((region, dict(nsites=nsites, updater_kwargs=upd, **rkws)))
        if len(region) == 2 and j < len(basic) - 1:
            rev = dict(upd, time_step=-upd["time_step"])
            sweep.append(([region[-1]], dict(updater_kwargs=rev, **rkws)))
    if not forward:
        sweep = [(list(reversed(r)), k) for (r, k) in reversed(sweep)]
    return sweep


def tdvp_regions(g: G, time_step, updater_kwargs, tdvp_order, nsites, **kws):
    plan = []
    for step, weight in enumerate(tdvp_sub_time_steps(tdvp_order), start=1):
        plan += first_order_sweep(g, weight * time_step, step % 2 == 1, updater_kwargs, nsites, **kws)
    return plan


# ----------------------------------------------------------------------------
# Tree tensor networks
# ----------------------------------------------------------------------------


class TTN:
    def __init__(self, g: G, tensors, ortho_region=None):
        self.g = g
        self.t = dict(tensors)
        self.stamp = {v: next(_stamp) for v in g.vertices}
        self.ortho_region = list(g.vertices) if ortho_region is None else list(ortho_region)

    def copy(self):
        c = TTN.__new__(TTN)
        c.g, c.t, c.stamp, c.ortho_region = self.g, dict(self.t), dict(self.stamp), list(self.ortho_region)
        return c

    def __getitem__(self, v):
        return self.t[v]

    def __setitem__(self, v, T):
        self.t[v] = T
        self.stamp[v] = next(_stamp)

    def linkind(self, u, v):
        return commonind(self.t[u], self.t[v])

    def maxlinkdim(self):
        return max((self.linkind(u, v).dim for (u, v) in self.g.edges), default=1)

    def linkdims(self):
        return {e: self.linkind(*e).dim for e in self.g.edges}

    def norm(self):
        return float(np.sqrt(abs(inner(self, self))))


def inner(a: TTN, b: TTN):
    """<a|b>: contract the two networks vertex by vertex in post order."""
    g = a.g
    root = g.default_root_vertex()
    parent = dict(post_order_dfs_edges(g, root))
    env = {}
    for v in post_order_dfs_vertices(g, root):
        T = a[v].dag().prime(*[a.linkind(v, u) for u in g.neighbors(v)])
        for u in g.neighbors(v):
            if u != parent.get(v):
                T = T * env.pop((u, v))
        T = T * b[v]
        if v in parent:
            env[(v, parent[v])] = T
        else:
            return T.scalar()
    raise RuntimeError("empty network")


def from_network(net, site_index=None, dtype=None):
    """Build oracle tensors from the plain data format of `networksolvers_gb300.models`.
    `site_index` maps vertex -> Index, shared between a state and its operator."""
    g = G(net.graph.vertices, net.graph.edges)
    site_index = {} if site_index is None else site_index
    links = {}
    tensors = {}
    kind = net.meta.get("kind", "state")
    for v in g.vertices:
        inds = []
        for leg, dim in zip(net.legs[v], net.tensors[v].shape):
            tag, x = leg
            if tag == "s":
                if x not in site_index:
                    site_index[x] = Index(dim, f"Site,n={x}")
                inds.append(site_index[x])
            elif tag == "sp":
                if x not in site_index:
                    site_index[x] = Index(dim, f"Site,n={x}")
                inds.append(site_index[x].prime())
            else:
                e = g.key(*x)
                if e not in links:
                    links[e] = Index(dim, ("Link" if tag == "l" else "OpLink") + f",e={e}")
                inds.append(links[e])
        data = net.tensors[v] if dtype is None else net.tensors[v].astype(dtype)
        tensors[v] = Tensor(data, inds)
    orth = net.meta.get("ortho_region", list(g.vertices))
    return (TTN(g, tensors, orth) if kind == "state" else (g, tensors)), site_index


def to_arrays(psi: TTN, net_like):
    """Export tensors in the plain leg order of `net_like` (links matched by edge)."""
    out = {}
    for v in psi.g.vertices:
        order = []
        for (tag, x) in net_like.legs[v]:
            if tag == "s":
                order.append([i for i in psi[v].inds if i.tags.startswith("Site")][0])
            else:
                u = x[0] if x[1] == v else x[1]
                order.append(psi.linkind(v, u))
        out[v] = psi[v].permute(order).data
    return out


def orthogonalize(psi: TTN, region):
    path = edge_sequence_between_regions(psi.g, psi.ortho_region, list(region))
    psi = psi.copy()
    for (s, d) in path:
        Q, R = linalg.qr(psi[s], uniqueinds(psi[s], psi[d]))
        psi[s] = Q
        psi[d] = R * psi[d]
    psi.ortho_region = list(region)
    return psi


class ProjTTN:
    """Environment cache of the projected operator."""

    def __init__(self, g: G, H: dict):
        self.g = g
        self.H = H
        self.pos = list(g.vertices)
        self.envs = {}  # (u,v) -> (Tensor, stamp, side)
        self._side = {}

    def side(self, u, v):
        if (u, v) not in self._side:
            self._side[(u, v)] = self.g.side(u, v)
        return self._side[(u, v)]

    def _valid(self, key, psi):
        if key not in self.envs:
            return False
        T, st, side = self.envs[key]
        return all(psi.stamp[x] <= st for x in side)

    def environment(self, psi: TTN, u, v):
        """Environment of directed edge u→v: subtree on u's side."""
        key = (u, v)
        if self._valid(key, psi):
            return self.envs[key][0]
        inc = [self.environment(psi, w, u) for w in self.g.neighbors(u) if w != v]
        A = psi[u]
        bra = A.dag().prime()
        T = A
        for E in inc:
            T = T * E
        T = T * self.H[u]
        T = T * bra
        stamp = next(_stamp)
        self.envs[key] = (T, stamp, self.side(u, v))
        return T

    def incident_edges(self, region):
        """Edges u→v with v in region, u outside (ITensorNetworks `incident_edges(P)`)."""
        out = []
        for v in region:
            for u in self.g.neighbors(v):
                if u not in region:
                    out.append((u, v))
        return out

    def position(self, psi: TTN, region):
        self.pos = list(region)
        self.psi = psi
        return self

    def position_edge(self, psi: TTN, edge):
        """A projected operator positioned on the bond (v1 → v2): its map uses the two
        environments of the bond.  Returned as a new view sharing the environment
        cache; the problem's own operator keeps its position (applyexp.jl:36)."""
        view = ProjTTN.__new__(ProjTTN)
        view.g, view.H, view.envs, view._side = self.g, self.H, self.envs, self._side
        view.pos = ("edge", edge)
        view.psi = psi
        return view


def optimal_map(P: ProjTTN, x: Tensor):
    """H_eff·x: contract the incident environments, the region's operator tensors and
    x (operator_map.jl:3-10), then drop primes; the result keeps x's index order."""
    psi = P.psi
    if isinstance(P.pos, tuple) and P.pos[0] == "edge":
        v1, v2 = P.pos[1]
        envs = [P.environment(psi, v1, v2), P.environment(psi, v2, v1)]
        ops = []
    else:
        region = P.pos
        envs = [P.environment(psi, u, v) for (u, v) in P.incident_edges(region)]
        ops = [P.H[v] for v in region]
    out = [i.prime() for i in x.inds]
    return contract(envs + ops + [x], out=out).noprime()
