"""Tree tensor networks on the device: graph, region plans, TTN, ProjTTN, optimal_map.

Mirrors the reference's host-side structure:
* region plans — region_plans/euler_tour.jl:4-48, euler_plans.jl:4-13,
  dfs_plans.jl:5-22, tdvp_region_plans.jl:1-44 (`default_root_vertex` of NamedGraphs
  is taken as the first leaf vertex in vertex order);
* `orthogonalize` — ITensorNetworks' gauge walk called at extracter.jl:6 (QR along the
  post-order edges of the Steiner tree joining the old and new regions);
* `ProjTTN` — ITensorNetworks' environment cache used by optimal_map
  (operator_map.jl:3-10) and `position` (extracter.jl:14): one environment per
  directed edge, recomputed when a tensor on its side changed;
* `LinearMap` — `x -> optimal_map(P, x)` as a device linear map (nsg_linmap), so
  the Krylov solvers run without returning to Python between applications.
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from . import _native as N
from .itensors import (DTensor, Index, contract, uniqueinds, commonind, qr)

_stamp = itertools.count(1)


# ----------------------------------------------------------------------------
# graph and plans
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
        self._side = {}

    @classmethod
    def from_graph(cls, g):
        return cls(g.vertices, g.edges)

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
        if (u, v) not in self._side:
            seen, stack = {u}, [u]
            while stack:
                x = stack.pop()
                for y in self.adjn[x]:
                    if y not in seen and not (x == u and y == v):
                        seen.add(y)
                        stack.append(y)
            self._side[(u, v)] = frozenset(seen)
        return self._side[(u, v)]


def post_order_dfs_vertices(g, root, allowed=None):
    out, seen = [], {root}
    stack = [(root, iter(g.neighbors(root)))]
    while stack:
        v, it = stack[-1]
        nxt = None
        for u in it:
            if (allowed is None or u in allowed) and u not in seen:
                nxt = u
                break
        if nxt is None:
            out.append(v)
            stack.pop()
        else:
            seen.add(nxt)
            stack.append((nxt, iter(g.neighbors(nxt))))
    return out


def post_order_dfs_edges(g, root, allowed=None):
    parent, seen, order = {root: None}, {root}, []
    stack = [(root, iter(g.neighbors(root)))]
    while stack:
        v, it = stack[-1]
        nxt = None
        for u in it:
            if (allowed is None or u in allowed) and u not in seen:
                nxt = u
                break
        if nxt is None:
            order.append(v)
            stack.pop()
        else:
            seen.add(nxt)
            parent[nxt] = v
            stack.append((nxt, iter(g.neighbors(nxt))))
    return [(v, parent[v]) for v in order if parent[v] is not None]


def steiner_tree(g, terminals):
    keep, terms = set(g.vertices), set(terminals)
    changed = True
    while changed:
        changed = False
        for v in list(keep):
            if v not in terms and sum(1 for u in g.neighbors(v) if u in keep) <= 1:
                keep.discard(v)
                changed = True
    return keep


def edge_sequence_between_regions(g, region1, region2):
    if set(region1) == set(region2):
        return []
    st = steiner_tree(g, list(region1) + list(region2))
    path = post_order_dfs_edges(g, region2[0], allowed=st)
    return [(s, d) for (s, d) in path if not (s in region2 and d in region2)]


def euler_tour_edges(g, start):
    adj = {v: [] for v in g.vertices}
    for (s, d) in g.edges_sorted():
        adj[s].append(d)
        adj[d].append(s)
    visited, tour, stack = set(), [], [start]
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


def euler_tour_vertices(g, start):
    edges = euler_tour_edges(g, start)
    return [edges[0][0]] + [e[1] for e in edges] if edges else []


def euler_sweep(g, nsites, root_vertex=None, **sweep_kwargs):
    root = g.default_root_vertex() if root_vertex is None else root_vertex
    if nsites == 1:
        return [([v], dict(sweep_kwargs)) for v in euler_tour_vertices(g, root)]
    return [([s, d], dict(sweep_kwargs)) for (s, d) in euler_tour_edges(g, root)]


def post_order_dfs_plan(g, nsites, root_vertex=None, **sweep_kwargs):
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


def first_order_sweep(g, time_step, forward, updater_kwargs, nsites, **kws):
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


def tdvp_regions(g, time_step, updater_kwargs, tdvp_order, nsites, **kws):
    plan = []
    for step, weight in enumerate(tdvp_sub_time_steps(tdvp_order), start=1):
        plan += first_order_sweep(g, weight * time_step, step % 2 == 1, updater_kwargs, nsites, **kws)
    return plan


# ----------------------------------------------------------------------------
# networks
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

    def linkdims(self):
        return {e: self.linkind(*e).dim for e in self.g.edges}

    def maxlinkdim(self):
        return max(self.linkdims().values(), default=1)

    def siteind(self, v):
        return [i for i in self.t[v].inds if i.tags.startswith("Site")][0]

    def to_numpy(self, net_like):
        """Tensors in the plain leg order of `net_like` (see models.Network)."""
        out = {}
        for v in self.g.vertices:
            order = []
            for (tag, x) in net_like.legs[v]:
                if tag == "s":
                    order.append(self.siteind(v))
                else:
                    u = x[0] if x[1] == v else x[1]
                    order.append(self.linkind(v, u))
            out[v] = self[v].permute(order).to_numpy() if list(self[v].inds) != order else self[v].to_numpy()
        return out


def from_network(net, site_index=None, ctx=None, dtype=None):
    """Upload a plain-data network (models.Network) to the device."""
    g = G.from_graph(net.graph)
    site_index = {} if site_index is None else site_index
    links, tensors = {}, {}
    kind = net.meta.get("kind", "state")
    for v in g.vertices:
        inds = []
        for (tag, x), dim in zip(net.legs[v], net.tensors[v].shape):
            if tag in ("s", "sp"):
                if x not in site_index:
                    site_index[x] = Index(dim, f"Site,n={x}")
                inds.append(site_index[x] if tag == "s" else site_index[x].prime())
            else:
                e = g.key(*x)
                if (tag, e) not in links:
                    links[(tag, e)] = Index(dim, ("Link" if tag == "l" else "OpLink") + f",e={e}")
                inds.append(links[(tag, e)])
        data = net.tensors[v] if dtype is None else net.tensors[v].astype(dtype)
        tensors[v] = DTensor.from_numpy(data, inds, ctx=ctx)
    if kind == "state":
        return TTN(g, tensors, net.meta.get("ortho_region")), site_index
    return (g, tensors), site_index


def inner(a: TTN, b: TTN):
    """<a|b> contracted vertex by vertex in post order."""
    g = a.g
    root = g.default_root_vertex()
    parent = dict(post_order_dfs_edges(g, root))
    env = {}
    for v in post_order_dfs_vertices(g, root):
        parts = [a[v].dag().prime(*[a.linkind(v, u) for u in g.neighbors(v)])]
        parts += [env.pop((u, v)) for u in g.neighbors(v) if u != parent.get(v)]
        parts.append(b[v])
        T = contract(parts)
        if v in parent:
            env[(v, parent[v])] = T
        else:
            x = T.to_numpy()
            return complex(x) if np.iscomplexobj(x) else float(x)
    raise RuntimeError("empty network")


def orthogonalize(psi: TTN, region):
    path = edge_sequence_between_regions(psi.g, psi.ortho_region, list(region))
    psi = psi.copy()
    for (s, d) in path:
        Q, R = qr(psi[s], uniqueinds(psi[s], psi[d]))
        psi[s] = Q
        psi[d] = R * psi[d]
    psi.ortho_region = list(region)
    return psi


class ProjTTN:
    """Environment cache of the projected operator (device tensors)."""

    def __init__(self, g: G, H: dict):
        self.g = g
        self.H = H
        self.pos = list(g.vertices)
        self.envs = {}
        self.psi = None

    def _valid(self, key, psi):
        e = self.envs.get(key)
        if e is None:
            return False
        T, st = e
        return all(psi.stamp[x] <= st for x in self.g.side(*key))

    def environment(self, psi: TTN, u, v):
        key = (u, v)
        if self._valid(key, psi):
            return self.envs[key][0]
        inc = [self.environment(psi, w, u) for w in self.g.neighbors(u) if w != v]
        A = psi[u]
        bra = A.dag().prime()
        # the bond index of A toward v: not its site index, not a link to another neighbour
        # (psi[v] may temporarily carry a different bond index, as in the 1-site TDVP
        # back-evolution where psi[u] = Q from a fresh QR)
        others = {psi.linkind(u, w) for w in self.g.neighbors(u) if w != v}
        site = psi.siteind(u)
        lk = [i for i in A.inds if i != site and i not in others][0]
        # output order [link', oplink, link] — the layout the chain kernels read
        hl = commonind(self.H[u], self.H[v])
        T = contract([A] + inc + [self.H[u], bra], out=[lk.prime(), hl, lk])
        self.envs[key] = (T, next(_stamp))
        return T

    def incident_edges(self, region):
        return [(u, v) for v in region for u in self.g.neighbors(v) if u not in region]

    def position(self, psi: TTN, region):
        self.pos = list(region)
        self.psi = psi
        return self

    def position_edge(self, psi: TTN, edge):
        view = ProjTTN.__new__(ProjTTN)
        view.g, view.H, view.envs = self.g, self.H, self.envs
        view.pos = ("edge", edge)
        view.psi = psi
        return view

    def map_tensors(self):
        psi = self.psi
        if isinstance(self.pos, tuple) and self.pos[0] == "edge":
            v1, v2 = self.pos[1]
            return [self.environment(psi, v1, v2), self.environment(psi, v2, v1)]
        envs = [self.environment(psi, u, v) for (u, v) in self.incident_edges(self.pos)]
        return envs + [self.H[v] for v in self.pos]


class LinearMap:
    """x -> optimal_map(P, x) (operator_map.jl:3-10) as a device linear map whose
    output keeps x's index order (noprime)."""

    def __init__(self, P: ProjTTN, x_inds):
        self.x_inds = tuple(x_inds)
        fixed = P.map_tensors()
        ctx = fixed[0].ctx
        self.ctx = ctx
        lab = {}
        for t in fixed:
            for i in t.inds:
                lab.setdefault(i, len(lab))
        for i in self.x_inds:
            lab.setdefault(i, len(lab))
            lab.setdefault(i.prime(), len(lab))
        dtype = N.C128 if any(t.is_complex() for t in fixed) else N.F64
        self.dtype = dtype
        self.fixed = fixed  # keep storages alive
        handles = (C.c_void_p * len(fixed))(*[t.st.h for t in fixed])
        flat = [lab[i] for t in fixed for i in t.inds]
        labels = (C.c_int32 * len(flat))(*flat)
        conj = (C.c_int * len(fixed))(*[int(t.conj) for t in fixed])
        xl = (C.c_int32 * len(self.x_inds))(*[lab[i] for i in self.x_inds])
        yl = (C.c_int32 * len(self.x_inds))(*[lab[i.prime()] for i in self.x_inds])
        h = C.c_void_p()
        ctx.check(ctx.L.nsg_linmap_create(ctx.h, len(fixed), handles, labels, conj, len(self.x_inds), xl, yl,
                                          C.byref(h)))
        self.h = h

    def flops(self):
        f = C.c_double()
        self.ctx.check(self.ctx.L.nsg_linmap_flops(self.h, C.byref(f)))
        return f.value

    def __call__(self, x: DTensor):
        y = DTensor.zeros(self.x_inds, x.dtype, ctx=self.ctx)
        xx = x if tuple(x.inds) == self.x_inds and not x.conj else x.permute(self.x_inds)
        self.ctx.check(self.ctx.L.nsg_linmap_apply(self.ctx.h, self.h, xx.st.h, y.st.h))
        return y

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.L.nsg_linmap_release(self.ctx.h, self.h)
        except Exception:
            pass
        self.h = None
