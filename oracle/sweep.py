"""The sweep: problems, extract/update/insert plugins and drivers (test infrastructure).

Follows, in order: iterators.jl:5-104 (SweepIterator/RegionIterator,
region_iterator_action), sweep_solve.jl:12-40, eigsolve.jl:4-76,
applyexp.jl:4-103, extracter.jl:3-17, inserter.jl:3-33, subspace/subspace.jl:8-48,
subspace/densitymatrix.jl:5-74, truncation_parameters.jl:1-14.
"""
from __future__ import annotations

import math

import numpy as np

from .tensor import Tensor, commonind, uniqueinds
from . import linalg, krylov
from .network import (TTN, ProjTTN, from_network, orthogonalize, optimal_map,
                      euler_sweep, tdvp_regions, edge_sequence_between_regions)


# ----------------------------------------------------------------------------
# truncation_parameters.jl:1-14
# ----------------------------------------------------------------------------


def get_or_last(x, i):
    if np.isscalar(x) or x is None:
        return x
    x = list(x)
    return x[-1] if i >= len(x) else x[i - 1]


def truncation_parameters(sweep, cutoff=0.0, maxdim=None, mindim=1):
    return dict(cutoff=get_or_last(cutoff, sweep), mindim=get_or_last(mindim, sweep),
                maxdim=get_or_last(maxdim, sweep))


# ----------------------------------------------------------------------------
# Problems and iterators
# ----------------------------------------------------------------------------


class EigsolveProblem:
    def __init__(self, state, operator):
        self.state, self.operator, self.eigenvalue = state, operator, math.inf


class ApplyExpProblem:
    def __init__(self, state, operator):
        self.state, self.operator, self.current_time = state, operator, 0.0


class RegionIterator:
    def __init__(self, problem, plan):
        self.problem, self.plan, self.which = problem, plan, 0

    @property
    def current_region(self):
        return self.plan[self.which][0]

    @property
    def next_region(self):
        return None if self.which == len(self.plan) - 1 else self.plan[self.which + 1][0]

    @property
    def previous_region(self):
        return None if self.which == 0 else self.plan[self.which - 1][0]


# ----------------------------------------------------------------------------
# Plugins
# ----------------------------------------------------------------------------


def _linmap(P, inds):
    return lambda x: optimal_map(P, Tensor(x, inds)).data


def extracter(problem, R, sweep, trunc=None, subspace_algorithm=None, **kws):
    trunc = truncation_parameters(sweep, **(trunc or {}))
    region = R.current_region
    psi = orthogonalize(problem.state, region)
    local = psi[region[0]]
    for v in region[1:]:
        local = local * psi[v]
    problem.state = psi
    problem, local = subspace_expand(problem, local, R, subspace_algorithm, trunc=trunc, **kws)
    problem.operator.position(problem.state, region)
    return problem, local


def subspace_expand(problem, local, R, algorithm, trunc, expansion_factor=1.5,
                    max_expand=None, north_pass=1, **kws):
    if algorithm is None:
        return problem, local
    if algorithm != "densitymatrix":
        raise ValueError("Subspace expansion (subspace_expand!) not defined for requested "
                         "combination of subspace_algorithm and problem types")
    region = R.current_region
    P = problem.operator
    psi = problem.state.copy()
    prev = [v for v in (P.pos if isinstance(P.pos, list) else []) if v not in region]
    if len(prev) != 1:
        return problem, local
    pv = prev[0]
    A = psi[pv]
    nxt = [v for v in region if commonind(psi[v], A) is not None]
    if not nxt:
        return problem, local
    nv = nxt[0]
    C = psi[nv]
    a = commonind(A, C)
    basis_size = int(np.prod([i.dim for i in uniqueinds(A, C)]))
    expand = compute_expansion(a.dim, basis_size, expansion_factor, max_expand, trunc["maxdim"])
    if expand <= 0:
        return problem, local
    tr = dict(trunc, maxdim=expand)
    # sqrt_rho = A · (environments of P not touching the region) · H[prev]
    sqrt_rho = A
    for (u, v) in P.incident_edges(P.pos):
        if u in region or v in region:
            continue
        sqrt_rho = sqrt_rho * P.environment(P.psi, u, v)
    sqrt_rho = sqrt_rho * P.H[pv]
    Ap = A.prime()
    for _ in range(north_pass):
        sqrt_rho = sqrt_rho - Ap * (Ap.dag() * sqrt_rho)
    rho = sqrt_rho * sqrt_rho.noprime().dag()
    ket = uniqueinds(A, C)
    D, U, u = linalg.eigen_hermitian(rho, ket, **tr)
    Apa = A.prime(a)
    for _ in range(north_pass):
        U = U - Apa * (Apa.dag() * U)
    if (U.dag() * A).norm() > 1e-10:
        return problem, local
    Ax, ax = linalg.directsum(A, a, U, u)
    expander = Ax.dag() * A
    psi[pv] = Ax
    psi[nv] = expander * C
    local = expander * local
    problem.state = psi
    return problem, local


def compute_expansion(current_dim, basis_size, expansion_factor=1.5, max_expand=None, maxdim=None):
    e = math.ceil(expansion_factor * current_dim)
    if max_expand is not None:
        e = min(max_expand, e)
    e = min(basis_size - current_dim, e)
    if maxdim is not None:
        e = min(maxdim - current_dim, e)
    return max(0, e)


def eigsolve_solver(linmap, init, which_eigval="SR", ishermitian=True, tol=1e-14,
                    krylovdim=3, maxiter=1, verbosity=0, eager=False, **kws):
    return krylov.eigsolve_lanczos(linmap, init, krylovdim=krylovdim, maxiter=maxiter, tol=tol)


def exponentiate_solver(linmap, time, init, krylovdim=30, maxiter=100, verbosity=0,
                        tol=1e-12, ishermitian=True, issymmetric=True, eager=True, **kws):
    return krylov.exponentiate(linmap, time, init, krylovdim=krylovdim, maxiter=maxiter, tol=tol)


def runge_kutta_solver(linmap, time, init, order=4, **kws):
    return krylov.runge_kutta_solver(linmap, time, init, order=order)


def updater_eigsolve(problem, local, R, outputlevel=0, solver=eigsolve_solver, **kws):
    lam, x = solver(_linmap(problem.operator, local.inds), local.data, **kws)
    problem.eigenvalue = lam
    return problem, Tensor(x, local.inds)


def updater_applyexp(problem, local, R, nsites, time_step, solver=runge_kutta_solver,
                     outputlevel=0, **kws):
    x, info = solver(_linmap(problem.operator, local.inds), time_step, local.data, **kws)
    local = Tensor(x, local.inds)
    if nsites == 1:
        cur, nxt = R.current_region, R.next_region
        if nxt is not None and nxt != cur:
            v1, v2 = edge_sequence_between_regions(problem.state.g, cur, nxt)[0]
            psi = problem.state.copy()
            Q, Rt = linalg.qr(local, uniqueinds(local, psi[v2]))
            psi[v1] = Q
            P = problem.operator.position_edge(psi, (v1, v2))
            r, _ = solver(_linmap(P, Rt.inds), -time_step, Rt.data, **kws)
            local = psi[v1] * Tensor(r, Rt.inds)
    problem.current_time = problem.current_time + time_step
    return problem, local


def inserter(problem, local, R, sweep, normalize=False, set_orthogonal_region=True,
             trunc=None, **kws):
    trunc = truncation_parameters(sweep, **(trunc or {}))
    region = R.current_region
    psi = problem.state.copy()
    info = {}
    if len(region) == 1:
        C = local
    elif len(region) == 2:
        U, C, err, spec, gap = linalg.factorize(local, list(psi[region[0]].inds), return_gap=True, **trunc)
        psi[region[0]] = U
        info = dict(truncerr=err, newdim=U.inds[-1].dim, cut_gap=gap)
    else:
        raise ValueError(f"Region of length {len(region)} not currently supported")
    v = region[-1]
    psi[v] = C
    if set_orthogonal_region:
        psi.ortho_region = [v]
    if normalize:
        psi[v] = psi[v] / psi[v].norm()
    problem.state = psi
    problem.last_insert = info
    return problem


# ----------------------------------------------------------------------------
# Driver: iterators.jl:81-100 + sweep_solve.jl:12-40
# ----------------------------------------------------------------------------


def region_iterator_action(problem, R, updater, extracter_kwargs=None, updater_kwargs=None,
                           inserter_kwargs=None, sweep=1, **kws):
    # Julia keyword splatting merges NamedTuples with the later one winning
    problem, local = extracter(problem, R, **{**dict(extracter_kwargs or {}), "sweep": sweep, **kws})
    problem, local = updater(problem, local, R, **{**dict(updater_kwargs or {}), **kws})
    problem = inserter(problem, local, R, **{"sweep": sweep, **dict(inserter_kwargs or {}), **kws})
    return problem


def sweep_solve(problem, plans, updater, region_callback=None, sweep_callback=None):
    for sweep, plan in enumerate(plans, start=1):
        R = RegionIterator(problem, plan)
        for k, (region, rkws) in enumerate(plan):
            R.which = k
            kws = dict(rkws)
            kws.pop("sweep", None)
            problem = region_iterator_action(problem, R, updater, sweep=sweep, **kws)
            if region_callback is not None:
                region_callback(problem, sweep=sweep, region=region, which=k)
        if sweep_callback is not None:
            sweep_callback(problem, sweep=sweep)
    return problem


def _prepare(H_net, psi_net):
    psi, sites = from_network(psi_net)
    (g, Ht), _ = from_network(H_net, site_index=sites)
    if np.iscomplexobj(psi_net.tensors[next(iter(psi_net.tensors))]) or np.iscomplexobj(
            H_net.tensors[next(iter(H_net.tensors))]):
        for v in list(Ht):
            Ht[v] = Tensor(Ht[v].data.astype(np.complex128), Ht[v].inds)
        for v in list(psi.t):
            psi.t[v] = Tensor(psi.t[v].data.astype(np.complex128), psi.t[v].inds)
    return psi, ProjTTN(psi.g, Ht)


def dmrg(H_net, psi_net, nsweeps, nsites=1, extracter_kwargs=None, updater_kwargs=None,
         inserter_kwargs=None, root_vertex=None, region_callback=None, sweep_callback=None,
         outputlevel=0):
    """eigsolve(H, ψ0; nsweeps, nsites, ...) → (eigenvalue, state) — eigsolve.jl:45-76."""
    psi, P = _prepare(H_net, psi_net)
    prob = EigsolveProblem(psi, P)
    kw = dict(extracter_kwargs=extracter_kwargs, updater_kwargs=updater_kwargs,
              inserter_kwargs=inserter_kwargs, outputlevel=outputlevel)
    plans = [euler_sweep(psi.g, nsites, root_vertex=root_vertex, **kw) for _ in range(nsweeps)]
    prob = sweep_solve(prob, plans, updater_eigsolve, region_callback, sweep_callback)
    return prob.eigenvalue, prob.state


eigsolve = dmrg


def applyexp(H_net, psi_net, exponents, nsites=1, tdvp_order=4, extracter_kwargs=None,
             updater_kwargs=None, inserter_kwargs=None, root_vertex=None, region_callback=None,
             sweep_callback=None, outputlevel=0, init=None):
    """applyexp(H, ψ0, exponents; ...) — applyexp.jl:62-89: one sweep per time step,
    time steps = diff([0, exponents...])."""
    if init is None:
        psi, P = _prepare(H_net, psi_net)
    else:
        psi, P = init
    prob = ApplyExpProblem(psi, P)
    # diff([0.0, exponents...])[2:end]: the first difference is dropped (applyexp.jl:74)
    steps = np.diff(np.concatenate([[0.0], np.asarray(exponents, dtype=np.complex128)]))[1:]
    plans = []
    for t in steps:
        plans.append(tdvp_regions(psi.g, t, updater_kwargs=dict(updater_kwargs or {}),
                                  tdvp_order=tdvp_order, nsites=nsites, root_vertex=root_vertex,
                                  extracter_kwargs=extracter_kwargs, inserter_kwargs=inserter_kwargs,
                                  outputlevel=outputlevel))
    prob = sweep_solve(prob, plans, updater_applyexp, region_callback, sweep_callback)
    return prob.state


def tdvp(H_net, psi_net, time_points, **kws):
    """tdvp — applyexp.jl:93-103 with exponents -i·t."""
    return applyexp(H_net, psi_net, [-1j * t for t in time_points], **kws)
