"""Two-site DMRG on a chain with one fused library call per region.

The same algorithm as `eigsolve(...; nsites=2)` on a chain graph (eigsolve.jl:45-76 with
the Euler-tour plan, euler_plans.jl:4-13: regions (1,2), (2,3), ..., (N-1,N), then (N,N-1),
..., (2,1) per sweep), without subspace expansion: every region step is one
`nsg_region_step` call (product, Lanczos, truncated factorization) plus one environment
contraction, so the host work per region is a handful of calls instead of the general
driver's index bookkeeping.  This is the driver the solve pool uses for chain jobs: its
host time per region is small enough for many solves to share one interpreter.

The initial gauge walk toward the first region is the general one (`orthogonalize`), so
the two drivers start from the same tensors and agree to rounding (tested).
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .itensors import DTensor, Index, contract
from .network import from_network, orthogonalize
from .sweep import get_or_last, region_step


def _pad3(arr, j, n):
    """State tensor of vertex j in [left, site, right] order with dim-1 boundary links."""
    if n == 1:
        return arr.reshape(1, -1, 1)
    if j == 1:
        return np.ascontiguousarray(arr.T)[None, :, :]   # [link, site] -> [1, site, link]
    if j == n:
        return arr[:, :, None]
    return arr


def _pad_op(arr, j, n):
    """Operator tensor of vertex j in [left, s', s, right] order with dim-1 boundary links."""
    if n == 1:
        return arr[None, :, :, None]
    if j == 1:
        return np.ascontiguousarray(arr.transpose(1, 2, 0))[None]   # [w, s', s] -> [1, s', s, w]
    if j == n:
        return arr[:, :, :, None]
    return arr


def dmrg_chain(H, psi0, nsweeps, maxdim=None, cutoff=0.0, mindim=1, krylovdim=3, maxiter=1, tol=1e-14, ctx=None,
               region_callback=None):
    """Ground state of the chain operator H (models.Network) from psi0 (models.Network on
    the same chain_graph, vertices 1..N).  `maxdim`, `cutoff`, `mindim` are scalars or
    per-sweep lists (the last entry repeats, truncation_parameters.jl:7-14).
    Returns (energy, {vertex: numpy tensor in psi0's leg order}, records) with records =
    [(sweep, region index, energy, new bond dimension), ...]."""
    ctx = ctx or N.default_context()
    g = psi0.graph
    n = len(g.vertices)
    verts = sorted(g.vertices)
    if verts != list(range(1, n + 1)) or any(sorted(g.neighbors(v)) != [u for u in (v - 1, v + 1) if 1 <= u <= n]
                                             for v in verts):
        raise ValueError("dmrg_chain: psi0 must live on a chain graph with vertices 1..N")
    cplx = any(np.iscomplexobj(t) for t in list(H.tensors.values()) + list(psi0.tensors.values()))
    dt = np.complex128 if cplx else np.float64
    # the general gauge walk toward the first region, then the tensors in [left, site, right]
    psi, sites = from_network(psi0, ctx=ctx, dtype=dt if cplx else None)
    psi = orthogonalize(psi, [1, 2] if n > 1 else [1])
    host = psi.to_numpy(psi0)
    padded = {j: _pad3(host[j], j, n).astype(dt, copy=False) for j in verts}
    bond = {0: Index(1, "Link,left"), n: Index(1, "Link,right")}
    for j in range(1, n):
        bond[j] = Index(padded[j].shape[2], f"Link,l={j}")
    site = {j: Index(padded[j].shape[1], f"Site,n={j}") for j in verts}
    A = {j: DTensor.from_numpy(padded[j], [bond[j - 1], site[j], bond[j]], ctx=ctx) for j in verts}
    wdims = {0: 1, n: 1}
    W = {}
    for j in verts:
        Wj = _pad_op(H.tensors[j], j, n).astype(dt, copy=False)
        wdims[j] = Wj.shape[3]
        W[j] = Wj
    wl = {j: Index(wdims[j], f"OpLink,l={j}") for j in range(0, n + 1)}
    Wt = {j: DTensor.from_numpy(W[j], [wl[j - 1], site[j].prime(), site[j], wl[j]], ctx=ctx) for j in verts}
    one = np.ones((1, 1, 1), dtype=dt)
    Lenv = {0: DTensor.from_numpy(one, [bond[0].prime(), wl[0], bond[0]], ctx=ctx)}
    Renv = {n + 1: DTensor.from_numpy(one, [bond[n].prime(), wl[n], bond[n]], ctx=ctx)}

    def left_env(j):   # sites 1..j: [a_j', w_j, a_j]
        a = A[j]
        return contract([Lenv[j - 1], a, Wt[j], a.dag().prime()], out=[bond[j].prime(), wl[j], bond[j]])

    def right_env(j):  # sites j..N: [a_{j-1}', w_{j-1}, a_{j-1}]
        a = A[j]
        return contract([Renv[j + 1], a, Wt[j], a.dag().prime()], out=[bond[j - 1].prime(), wl[j - 1], bond[j - 1]])

    for j in range(n, 2, -1):
        Renv[j] = right_env(j)
    records = []
    energy = None
    for sweep in range(1, nsweeps + 1):
        md = get_or_last(maxdim, sweep) if maxdim is not None else None
        co = get_or_last(cutoff, sweep)
        mi = get_or_last(mindim, sweep)
        regions = [(j, 0) for j in range(1, n)] + [(j, 1) for j in range(n - 1, 0, -1)]
        for k, (j, direction) in enumerate(regions):
            energy, left, right, info = region_step(Lenv[j - 1], Wt[j], Wt[j + 1], Renv[j + 2], A[j], A[j + 1],
                                                    direction=direction, krylovdim=krylovdim, maxiter=maxiter,
                                                    tol=tol, cutoff=co, maxdim=md, mindim=mi)
            link = left.inds[2]
            bond[j] = link
            A[j] = DTensor(left.st, [bond[j - 1], site[j], link])
            A[j + 1] = DTensor(right.st, [link, site[j + 1], bond[j + 1]])
            if direction == 0 and j < n - 1:
                Lenv[j] = left_env(j)
            elif direction == 1 and j > 1:
                Renv[j + 1] = right_env(j + 1)
            records.append((sweep, k, energy, info["newdim"]))
            if region_callback is not None:
                region_callback(sweep, k, energy, info)
    out = {}
    for j in verts:
        t = A[j].to_numpy()
        if n == 1:
            t = t[0, :, 0]
        elif j == 1:
            t = t[0].T          # [site, link] -> [link, site]
        elif j == n:
            t = t[:, :, 0]
        out[j] = t
    return energy, out, records
