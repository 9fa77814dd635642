"""The reference's sweep API on the device: problems, plugins, solvers and drivers.

Same names, arguments and control flow as NetworkSolvers.jl:
  eigsolve/dmrg          eigsolve.jl:45-76      applyexp/tdvp      applyexp.jl:62-103
  EigsolveProblem        eigsolve.jl:4-8        ApplyExpProblem    applyexp.jl:4-8
  region_iterator_action iterators.jl:81-100    sweep_solve        sweep_solve.jl:12-40
  extracter              extracter.jl:3-17      inserter           inserter.jl:3-33
  updater (eigsolve)     eigsolve.jl:14-28      updater (applyexp) applyexp.jl:18-48
  subspace_expand        subspace/subspace.jl:8-48, subspace/densitymatrix.jl:5-74
  truncation_parameters  truncation_parameters.jl:1-14
  eigsolve_solver / exponentiate_solver / runge_kutta_solver   local_solvers/*.jl
Every numerical step runs through libnsg (include/nsg.h); the Python layer only
keeps index bookkeeping, plans and control flow, as the Julia layer does.
"""
from __future__ import annotations

import ctypes as C
import math
from contextlib import contextmanager

import numpy as np

from . import _native as N
from .itensors import (DTensor, commonind, uniqueinds, factorize, qr, eigen_hermitian, directsum)
from .network import (TTN, ProjTTN, LinearMap, from_network, orthogonalize, euler_sweep,
                      tdvp_regions, edge_sequence_between_regions)


# ----------------------------------------------------------------------------
# truncation_parameters.jl
# ----------------------------------------------------------------------------


def get_or_last(x, i):
    if x is None or np.isscalar(x):
        return x
    x = list(x)
    return x[-1] if i >= len(x) else x[i - 1]


def truncation_parameters(sweep, cutoff=0.0, maxdim=None, mindim=1):
    return dict(cutoff=get_or_last(cutoff, sweep), mindim=get_or_last(mindim, sweep),
                maxdim=get_or_last(maxdim, sweep))


# ----------------------------------------------------------------------------
# problems / iterators
# ----------------------------------------------------------------------------


class EigsolveProblem:
    def __init__(self, state, operator):
        self.state, self.operator, self.eigenvalue = state, operator, math.inf
        self.last_insert = {}


class ApplyExpProblem:
    def __init__(self, state, operator):
        self.state, self.operator, self.current_time = state, operator, 0.0
        self.last_insert = {}


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
# local solvers (local_solvers/*.jl) on the device
# ----------------------------------------------------------------------------


def _vec(op: LinearMap, init: DTensor):
    x = init if tuple(init.inds) == op.x_inds and not init.conj else init.permute(op.x_inds)
    return x.copy()


def eigsolve_solver(operator, init, howmany=1, which_eigval="SR", ishermitian=True, tol=1e-14, krylovdim=3,
                    maxiter=1, verbosity=0, eager=False, **kws):
    x = _vec(operator, init)
    ctx = x.ctx
    lam, nops = C.c_double(), C.c_int()
    ctx.check(ctx.L.nsg_eigsolve(ctx.h, operator.h, x.st.h, int(krylovdim), int(maxiter), float(tol),
                                 C.byref(lam), C.byref(nops)))
    return lam.value, x


def exponentiate_solver(operator, time, init, krylovdim=30, maxiter=100, verbosity=0, tol=1e-12,
                        ishermitian=True, issymmetric=True, eager=True, **kws):
    x = _vec(operator, init)
    ctx = x.ctx
    t = complex(time)
    conv, nops = C.c_int(), C.c_int()
    ctx.check(ctx.L.nsg_exponentiate(ctx.h, operator.h, t.real, t.imag, x.st.h, int(krylovdim), int(maxiter),
                                     float(tol), C.byref(conv), C.byref(nops)))
    return x, dict(converged=bool(conv.value), numops=nops.value)


def runge_kutta_solver(operator, time, init, order=4, **kws):
    x = _vec(operator, init)
    ctx = x.ctx
    t = complex(time)
    ctx.check(ctx.L.nsg_runge_kutta(ctx.h, operator.h, t.real, t.imag, x.st.h, int(order)))
    return x, {}


# ----------------------------------------------------------------------------
# plugins
# ----------------------------------------------------------------------------


def extracter(problem, region_iterator, sweep, trunc=None, subspace_algorithm=None, **kws):
    trunc = truncation_parameters(sweep, **(trunc or {}))
    region = region_iterator.current_region
    psi = orthogonalize(problem.state, region)
    local = psi[region[0]]
    for v in region[1:]:
        local = local * psi[v]
    problem.state = psi
    problem, local = subspace_expand(problem, local, region_iterator, subspace_algorithm, trunc=trunc, **kws)
    problem.operator.position(problem.state, region)
    return problem, local


def compute_expansion(current_dim, basis_size, expansion_factor=1.5, max_expand=None, maxdim=None):
    e = math.ceil(expansion_factor * current_dim)
    if max_expand is not None:
        e = min(max_expand, e)
    e = min(basis_size - current_dim, e)
    if maxdim is not None:
        e = min(maxdim - current_dim, e)
    return max(0, e)


def subspace_expand(problem, local, region_iterator, algorithm, trunc, expansion_factor=1.5, max_expand=None,
                    north_pass=1, **kws):
    if algorithm is None:
        return problem, local
    if algorithm != "densitymatrix":
        raise ValueError("Subspace expansion (subspace_expand!) not defined for requested combination of "
                         "subspace_algorithm and problem types")
    region = region_iterator.current_region
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
    Cn = psi[nv]
    a = commonind(A, Cn)
    basis_size = int(np.prod([i.dim for i in uniqueinds(A, Cn)]))
    expand = compute_expansion(a.dim, basis_size, expansion_factor, max_expand, trunc["maxdim"])
    if expand <= 0:
        return problem, local
    tr = dict(trunc, maxdim=expand)
    # An orthonormal complement of A's columns, when the factorization that made A produced
    # one (its discarded eigenvectors; the inserter keeps the latest once an expansion has
    # run): eigen(rho) restricted to it is the same eigenproblem, of dimension
    # rows(A) - dim(a) instead of rows(A), since rho = X X^H with X = (1 - A A^H) sqrt_rho.
    basis = getattr(problem, "expansion_basis", None)
    if basis is None:
        problem.expansion_basis = basis = ()
    perp = basis[2] if (basis and basis[0] == pv and basis[1] is A.st and not A.conj) else None
    # the expansion's projections are checked against a 1e-10 orthogonality guard
    # (densitymatrix.jl:59): its contractions run at FP64 accuracy whatever the context's
    # mode (eight-slice tensor-core products in the split form, FP64 cores otherwise)
    ctx = A.ctx
    prec = ctx.precision
    ctx.set_precision("ozaki8" if prec in ("ozaki", "ozaki8") else "fp64")
    try:
        with _phase("subspace"):
            return _densitymatrix(problem, local, region, P, psi, pv, nv, A, Cn, a, tr, north_pass, perp)
    finally:
        ctx.set_precision(prec)


def _densitymatrix(problem, local, region, P, psi, pv, nv, A, Cn, a, tr, north_pass, perp=None):
    parts = [A]
    for (u, v) in P.incident_edges(P.pos):
        if u in region or v in region:
            continue
        parts.append(P.environment(P.psi, u, v))
    parts.append(P.H[pv])
    from .itensors import contract
    sqrt_rho = contract(parts)
    ket = uniqueinds(A, Cn)
    if perp is not None and {i.key() for i in perp.inds[:-1]} == {i.key() for i in ket}:
        # Y = Uperp^H sqrt_rho (Uperp^H A = 0 makes the projection redundant), R = Y Y^H,
        # eigenvectors Uperp Z
        q = perp.inds[-1]
        Y = perp.prime().dag() * sqrt_rho
        R = Y * Y.noprime().dag()
        D, Z, u = eigen_hermitian(R, [q], **tr)
        U = perp * Z
    else:
        Ap = A.prime()
        for _ in range(north_pass):
            sqrt_rho = sqrt_rho - Ap * (Ap.dag() * sqrt_rho)
        rho = sqrt_rho * sqrt_rho.noprime().dag()
        D, U, u = eigen_hermitian(rho, ket, **tr)
    Apa = A.prime(a)
    for _ in range(north_pass):
        U = U - Apa * (Apa.dag() * U)
    if (U.dag() * A).norm() > 1e-10:
        return problem, local
    Ax, ax = directsum(A, a, U, u)
    expander = Ax.dag() * A
    psi[pv] = Ax
    psi[nv] = expander * Cn
    local = expander * local
    problem.state = psi
    return problem, local


def updater_eigsolve(problem, local, region_iterator, outputlevel=0, solver=eigsolve_solver, **kws):
    lm = LinearMap(problem.operator, local.inds)
    problem.last_flops = lm.flops()
    lam, x = solver(lm, local, **kws)
    problem.eigenvalue = lam
    if outputlevel >= 2:
        print(f"  Region {region_iterator.current_region}: energy = {lam:.12f}")
    return problem, x


def updater_applyexp(problem, local, region_iterator, nsites, time_step, solver=runge_kutta_solver,
                     outputlevel=0, **kws):
    lm = LinearMap(problem.operator, local.inds)
    local, info = solver(lm, time_step, local, **kws)
    if nsites == 1:
        cur, nxt = region_iterator.current_region, region_iterator.next_region
        if nxt is not None and nxt != cur:
            v1, v2 = edge_sequence_between_regions(problem.state.g, cur, nxt)[0]
            psi = problem.state.copy()
            Q, R = qr(local, uniqueinds(local, psi[v2]))
            psi[v1] = Q
            Pe = problem.operator.position_edge(psi, (v1, v2))
            Rt, _ = solver(LinearMap(Pe, R.inds), -time_step, R, **kws)
            local = psi[v1] * Rt
    problem.current_time = problem.current_time + time_step
    return problem, local


def inserter(problem, local, region_iterator, sweep, normalize=False, set_orthogonal_region=True, trunc=None,
             **kws):
    trunc = truncation_parameters(sweep, **(trunc or {}))
    region = region_iterator.current_region
    psi = problem.state.copy()
    info = {}
    if len(region) == 1:
        Cn = local
    elif len(region) == 2:
        # once a densitymatrix expansion has run, keep the complement of U's columns for the
        # next region's expansion of this vertex
        basis = getattr(problem, "expansion_basis", None)
        U, Cn, info = factorize(local, list(psi[region[0]].inds), complement=basis is not None, **trunc)
        psi[region[0]] = U
        if basis is not None:
            perp = info.pop("complement", None)
            problem.expansion_basis = (region[0], U.st, perp) if perp is not None else ()
    else:
        raise ValueError(f"Region of length {len(region)} not currently supported")
    v = region[-1]
    psi[v] = Cn
    if set_orthogonal_region:
        psi.ortho_region = [v]
    if normalize:
        psi[v] = psi[v] / psi[v].norm()
    problem.state = psi
    problem.last_insert = info
    return problem


def region_step(L, W1, W2, R, psi1, psi2, direction=0, krylovdim=3, maxiter=1, tol=1e-14, cutoff=0.0, maxdim=None,
                mindim=1, tags="Link"):
    """One fused two-site region step (nsg_region_step): psi1·psi2, Lanczos on the H_eff of
    [L, R, W1, W2], truncated factorization — the extracter / updater / inserter of one
    chain region in a single library call.  Layout: L [a', wl, a], W1 [wl, s1', s1, wm],
    W2 [wm, s2', s2, wr], R [b', wr, b], psi1 [a, s1, c], psi2 [c, s2, b].  direction 0:
    the new left tensor is left-orthonormal; 1: the new right tensor is right-orthonormal.
    Returns (energy, left [a, s1, k], right [k, s2, b], info)."""
    from .itensors import Index, Storage
    ctx = psi1.ctx
    ts = [t.materialize() for t in (L, W1, W2, R, psi1, psi2)]
    U, Cc = C.c_void_p(), C.c_void_p()
    E, k, err = C.c_double(), C.c_int64(), C.c_double()
    md = -1 if maxdim is None else int(maxdim)
    ctx.check(ctx.L.nsg_region_step(ctx.h, *[t.st.h for t in ts], int(direction), int(krylovdim), int(maxiter),
                                    float(tol),
                                    float(cutoff), md, int(mindim), C.byref(U), C.byref(Cc), C.byref(E),
                                    C.byref(k), C.byref(err)))
    p1, p2 = ts[4], ts[5]
    link = Index(k.value, tags)
    dt = p1.dtype
    Ut = DTensor(Storage(ctx, U, dt, [p1.inds[0].dim, p1.inds[1].dim, k.value]), [p1.inds[0], p1.inds[1], link])
    Ct = DTensor(Storage(ctx, Cc, dt, [k.value, p2.inds[1].dim, p2.inds[2].dim]), [link, p2.inds[1], p2.inds[2]])
    return E.value, Ut, Ct, dict(newdim=k.value, truncerr=err.value)


# ----------------------------------------------------------------------------
# drivers
# ----------------------------------------------------------------------------


@contextmanager
def _phase(name):
    """Brackets a phase of the region step on the current context's stream while its
    per-phase timers run (Context.timers); nothing otherwise."""
    ctx = N.current_context()
    timing = ctx is not None and ctx.timing
    if timing:
        ctx.phase(name, True)
    try:
        yield
    finally:
        if timing:
            ctx.phase(name, False)


def region_iterator_action(problem, region_iterator, updater, extracter_kwargs=None, updater_kwargs=None,
                           inserter_kwargs=None, sweep=1, **kws):
    with _phase("extract"):
        problem, local = extracter(problem, region_iterator, **{**dict(extracter_kwargs or {}), "sweep": sweep, **kws})
    with _phase("krylov"):
        problem, local = updater(problem, local, region_iterator, **{**dict(updater_kwargs or {}), **kws})
    with _phase("factorize"):
        problem = inserter(problem, local, region_iterator, **{"sweep": sweep, **dict(inserter_kwargs or {}), **kws})
    return problem


def sweep_solve(problem, plans, updater, region_callback=None, sweep_callback=None, sweep_printer=None):
    nsweeps = len(plans)
    for sweep, plan in enumerate(plans, start=1):
        R = RegionIterator(problem, plan)
        for k, (region, rkws) in enumerate(plan):
            R.which = k
            kws = dict(rkws)
            kws.pop("sweep", None)
            problem = region_iterator_action(problem, R, updater, sweep=sweep, **kws)
            if region_callback is not None:
                region_callback(problem, sweep=sweep, region=region, which=k, nsweeps=nsweeps)
        if sweep_callback is not None:
            sweep_callback(problem, sweep=sweep, nsweeps=nsweeps)
        if sweep_printer is not None:
            sweep_printer(problem, sweep=sweep, nsweeps=nsweeps)
    return problem


def _prepare(H_net, psi_net, ctx=None):
    cplx = any(np.iscomplexobj(t) for t in list(H_net.tensors.values()) + list(psi_net.tensors.values()))
    dt = np.complex128 if cplx else None
    psi, sites = from_network(psi_net, ctx=ctx, dtype=dt)
    (g, Ht), _ = from_network(H_net, site_index=sites, ctx=ctx, dtype=dt)
    return psi, ProjTTN(psi.g, Ht)


def eigsolve_sweep_printer(problem, sweep, nsweeps, **kws):
    fmt = f"After sweep {sweep:02d}/{nsweeps} " if nsweeps >= 10 else f"After sweep {sweep}/{nsweeps} "
    print(fmt + f"eigenvalue={problem.eigenvalue:.12f} maxlinkdim={problem.state.maxlinkdim()}", flush=True)


def eigsolve(H, psi0, nsweeps, nsites=1, outputlevel=0, extracter_kwargs=None, updater_kwargs=None,
             inserter_kwargs=None, root_vertex=None, region_callback=None, sweep_callback=None, ctx=None,
             init=None):
    """`eigsolve(H, ψ0; nsweeps, nsites, ...)` → (eigenvalue, state); eigsolve.jl:45-76.
    H, ψ0: plain-data networks (models.Network) or, via `init`, a prepared (TTN, ProjTTN)."""
    psi, P = init if init is not None else _prepare(H, psi0, ctx)
    prob = EigsolveProblem(psi, P)
    kw = dict(extracter_kwargs=extracter_kwargs, updater_kwargs=updater_kwargs,
              inserter_kwargs=inserter_kwargs, outputlevel=outputlevel)
    plans = [euler_sweep(psi.g, nsites, root_vertex=root_vertex, **kw) for _ in range(nsweeps)]
    printer = eigsolve_sweep_printer if outputlevel >= 1 else None
    prob = sweep_solve(prob, plans, updater_eigsolve, region_callback, sweep_callback, printer)
    return prob.eigenvalue, prob.state


dmrg = eigsolve


def applyexp(H, psi0, exponents, nsites=1, tdvp_order=4, outputlevel=0, extracter_kwargs=None,
             updater_kwargs=None, inserter_kwargs=None, root_vertex=None, region_callback=None,
             sweep_callback=None, ctx=None, init=None):
    """`applyexp(H, ψ0, exponents; ...)` — one sweep per time step, steps = diff of the
    exponents with the first difference dropped (applyexp.jl:74)."""
    psi, P = init if init is not None else _prepare(H, psi0, ctx)
    prob = ApplyExpProblem(psi, P)
    steps = np.diff(np.concatenate([[0.0], np.asarray(exponents, dtype=np.complex128)]))[1:]
    plans = [tdvp_regions(psi.g, t, updater_kwargs=dict(updater_kwargs or {}), tdvp_order=tdvp_order,
                          nsites=nsites, root_vertex=root_vertex, extracter_kwargs=extracter_kwargs,
                          inserter_kwargs=inserter_kwargs, outputlevel=outputlevel) for t in steps]
    prob = sweep_solve(prob, plans, updater_applyexp, region_callback, sweep_callback)
    return prob.state


def tdvp(H, psi0, time_points, **kws):
    """`tdvp(H, ψ0, time_points)` with exponents −i·t (applyexp.jl:93-103)."""
    return applyexp(H, psi0, [-1j * t for t in time_points], **kws)
