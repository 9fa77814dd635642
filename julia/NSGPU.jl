# NSGPU.jl — the NetworkSolvers.jl plugins on the GB300 kernels of libnsg.so.
#
# NOT EXECUTED IN THIS REPOSITORY: neither the build machine nor the GPU machine has a
# Julia toolchain, so this module is written against the C ABI in include/nsg.h and the
# reference's plugin signatures but has never run.  The Python mirror in
# networksolvers_gb300/ (sweep.py, network.py, itensors.py) calls the same entry points
# through ctypes with the same control flow, and that is what the tests exercise.
#
# Usage (same drivers, region plans and keyword arguments as the reference):
#
#     using NetworkSolvers, NSGPU
#     ctx = NSGPU.Ctx(0)                       # one context (CUDA stream) per task
#     NSGPU.set_precision!(ctx, :ozaki)        # split form; :fp64 is the plain form
#     prob = NetworkSolvers.EigsolveProblem(; state=NSGPU.DeviceTTN(ctx, ψ0),
#                                             operator=NSGPU.DeviceProjTTN(ctx, H))
#     E, ψ = NetworkSolvers.eigsolve(prob; nsweeps, nsites=2, inserter_kwargs=(; trunc))
#     ψ_host = NSGPU.to_itensornetwork(ψ)
#
# The overrides below dispatch on the device types, so the reference's own
# region_iterator_action (iterators.jl:81-100) calls them unchanged:
#   extracter       extracter.jl:3-17         (gauge walk, region product, expansion, position)
#   updater         eigsolve.jl:14-28, applyexp.jl:18-48
#   inserter        inserter.jl:3-33
#   subspace_expand subspace/densitymatrix.jl:5-74
module NSGPU

import ITensors as it
import ITensorNetworks as itn
import NetworkSolvers as ns
using ITensors: ITensor, Index, inds, dim, prime, noprime, dag, commonind, uniqueinds, hascommoninds
using ConstructionBase: setproperties

const lib = joinpath(@__DIR__, "..", "networksolvers_gb300", "libnsg.so")

# ---------------------------------------------------------------------------
# context and status
# ---------------------------------------------------------------------------

mutable struct Ctx
  h::Ptr{Cvoid}
end
function Ctx(device::Integer=0; budget::Integer=0)
  r = Ref{Ptr{Cvoid}}(C_NULL)
  rc = @ccall lib.nsg_ctx_create(device::Cint, UInt64(budget)::UInt64, r::Ptr{Ptr{Cvoid}})::Cint
  rc == 0 || error("nsg_ctx_create failed with status $rc")
  c = Ctx(r[])
  finalizer(x -> (@ccall lib.nsg_ctx_destroy(x.h::Ptr{Cvoid})::Cint), c)
  return c
end
function check(c::Ctx, rc)
  rc == 0 && return nothing
  msg = unsafe_string(@ccall lib.nsg_last_error(c.h::Ptr{Cvoid})::Cstring)
  return error("nsg error $rc: $msg")
end
const PRECISION = Dict(:fp64 => 0, :tf32x3 => 1, :ozaki => 2, :ozaki8 => 3)
set_precision!(c::Ctx, p::Symbol) = check(c, @ccall lib.nsg_ctx_set_precision(c.h::Ptr{Cvoid}, PRECISION[p]::Cint)::Cint)
# pin one launch choice of the compiled-in tuning table for this context (measurement):
# :splitk => 1..64 K slices of small FP64 products, :tridiag => -1 (grid kernel) or a
# cluster size 2/4/8/16, :dc_leaf => divide-and-conquer leaf order 4..32; 0 returns to
# the table
const TUNING = Dict(:splitk => 0, :tridiag => 1, :dc_leaf => 2)
set_tuning!(c::Ctx, p::Symbol, v::Integer) =
  check(c, @ccall lib.nsg_ctx_set_tuning(c.h::Ptr{Cvoid}, TUNING[p]::Cint, Cint(v)::Cint)::Cint)
# per-phase device timers of the region step: the overrides below bracket their phases,
# the library brackets every H_eff application itself
const PHASES = (:extract, :subspace, :krylov, :heff, :factorize)
const TIMING = Ref(false)  # whether the overrides bracket their phases
function timers!(c::Ctx, on::Bool)
  check(c, @ccall lib.nsg_ctx_timers(c.h::Ptr{Cvoid}, Cint(on)::Cint)::Cint)
  TIMING[] = on
  return nothing
end
function phase(f, c::Ctx, p::Symbol)
  TIMING[] || return f()
  k = Cint(findfirst(==(p), PHASES) - 1)
  check(c, @ccall lib.nsg_ctx_phase(c.h::Ptr{Cvoid}, k::Cint, Cint(1)::Cint)::Cint)
  try
    return f()
  finally
    check(c, @ccall lib.nsg_ctx_phase(c.h::Ptr{Cvoid}, k::Cint, Cint(0)::Cint)::Cint)
  end
end
function timers(c::Ctx)
  n = zeros(UInt64, length(PHASES)); ms = zeros(Float64, length(PHASES))
  check(c, @ccall lib.nsg_get_timers(c.h::Ptr{Cvoid}, n::Ptr{UInt64}, ms::Ptr{Float64})::Cint)
  return Dict(p => (count=n[i], ms=ms[i]) for (i, p) in enumerate(PHASES))
end

# ---------------------------------------------------------------------------
# device tensors: an ITensor's dense storage is column-major in index order, the
# layout nsg.h expects; a DT keeps the indices beside the handle
# ---------------------------------------------------------------------------

mutable struct DT
  ctx::Ctx
  h::Ptr{Cvoid}
  inds::Vector{Index}
  cplx::Bool
end
function wrap(c::Ctx, h::Ptr{Cvoid}, is, cplx::Bool)
  t = DT(c, h, collect(is), cplx)
  finalizer(x -> (@ccall lib.nsg_tensor_release(x.ctx.h::Ptr{Cvoid}, x.h::Ptr{Cvoid})::Cint), t)
  return t
end
function upload(c::Ctx, T::ITensor)
  is = inds(T)
  A = Array(T, is...)
  cplx = eltype(A) <: Complex
  A = cplx ? ComplexF64.(A) : Float64.(A)
  dims = Int64[dim(i) for i in is]
  r = Ref{Ptr{Cvoid}}(C_NULL)
  check(c, @ccall lib.nsg_tensor_upload(c.h::Ptr{Cvoid}, Cint(cplx)::Cint, length(dims)::Cint, dims::Ptr{Int64},
                                        A::Ptr{Cvoid}, r::Ptr{Ptr{Cvoid}})::Cint)
  return wrap(c, r[], is, cplx)
end
function download(t::DT)
  A = Array{t.cplx ? ComplexF64 : Float64}(undef, Tuple(dim.(t.inds)))
  check(t.ctx, @ccall lib.nsg_tensor_download(t.ctx.h::Ptr{Cvoid}, t.h::Ptr{Cvoid}, A::Ptr{Cvoid})::Cint)
  return ITensor(A, t.inds...)
end
function norm(t::DT)
  r = Ref{Float64}()
  check(t.ctx, @ccall lib.nsg_norm(t.ctx.h::Ptr{Cvoid}, t.h::Ptr{Cvoid}, r::Ptr{Float64})::Cint)
  return r[]
end
function scale!(t::DT, s::Number)
  # y = 0 * y + s * y: axpby with x = y
  check(t.ctx, @ccall lib.nsg_axpby(t.ctx.h::Ptr{Cvoid}, 0.0::Float64, 0.0::Float64, t.h::Ptr{Cvoid},
                                    real(s)::Float64, imag(s)::Float64, t.h::Ptr{Cvoid})::Cint)
  return t
end

# ITensor index (id, prime level) -> int32 label of nsg_contract
label(i::Index) = Int32(mod(hash((it.id(i), it.plev(i))), 2^30))

# contract device tensors; the result's indices are the ones appearing once
function contract(c::Ctx, ts::Vector{DT}; conj::Vector{Bool}=fill(false, length(ts)))
  allinds = reduce(vcat, [t.inds for t in ts])
  out = [i for i in allinds if count(==(i), allinds) == 1]
  hs = [t.h for t in ts]
  lab = Int32[label(i) for i in allinds]
  cj = Cint[x for x in conj]
  ol = Int32[label(i) for i in out]
  r = Ref{Ptr{Cvoid}}(C_NULL)
  check(c, @ccall lib.nsg_contract(c.h::Ptr{Cvoid}, length(hs)::Cint, hs::Ptr{Ptr{Cvoid}}, lab::Ptr{Int32},
                                   cj::Ptr{Cint}, length(ol)::Cint, ol::Ptr{Int32}, r::Ptr{Ptr{Cvoid}})::Cint)
  return wrap(c, r[], out, any(t.cplx for t in ts))
end
function permute(t::DT, is)
  perm = Cint[findfirst(==(i), t.inds) - 1 for i in is]
  r = Ref{Ptr{Cvoid}}(C_NULL)
  check(t.ctx, @ccall lib.nsg_permute(t.ctx.h::Ptr{Cvoid}, t.h::Ptr{Cvoid}, perm::Ptr{Cint}, 0::Cint,
                                      r::Ptr{Ptr{Cvoid}})::Cint)
  return wrap(t.ctx, r[], collect(is), t.cplx)
end

# ---------------------------------------------------------------------------
# the linear map of optimal_map(P, ψ) (operator_map.jl:3-10): fixed tensors are the
# incident environments and the region's operator tensors; the result is noprime'd
# into ψ's shape
# ---------------------------------------------------------------------------

mutable struct LinMap
  ctx::Ctx
  h::Ptr{Cvoid}
end
function LinMap(c::Ctx, fixed::Vector{DT}, x_inds)
  hs = [f.h for f in fixed]
  lab = Int32[label(i) for f in fixed for i in f.inds]
  xl = Int32[label(i) for i in x_inds]
  yl = Int32[label(prime(i)) for i in x_inds]
  r = Ref{Ptr{Cvoid}}(C_NULL)
  check(c, @ccall lib.nsg_linmap_create(c.h::Ptr{Cvoid}, length(hs)::Cint, hs::Ptr{Ptr{Cvoid}}, lab::Ptr{Int32},
                                        C_NULL::Ptr{Cint}, length(xl)::Cint, xl::Ptr{Int32}, yl::Ptr{Int32},
                                        r::Ptr{Ptr{Cvoid}})::Cint)
  m = LinMap(c, r[])
  finalizer(x -> (@ccall lib.nsg_linmap_release(x.ctx.h::Ptr{Cvoid}, x.h::Ptr{Cvoid})::Cint), m)
  return m
end

# ---------------------------------------------------------------------------
# device state and projected operator
# ---------------------------------------------------------------------------

mutable struct DeviceTTN
  ctx::Ctx
  graph::Any                          # NamedGraph of the network
  t::Dict{Any,DT}                     # vertex => site tensor (permute_indices order)
  stamp::Dict{Any,Int}
  ortho_region::Vector{Any}
end
const STAMP = Ref(0)
nextstamp() = (STAMP[] += 1)
function DeviceTTN(c::Ctx, ψ)
  ψ = ns.permute_indices(ψ)
  g = itn.underlying_graph(ψ)
  t = Dict{Any,DT}(v => upload(c, ψ[v]) for v in itn.vertices(ψ))
  return DeviceTTN(c, g, t, Dict{Any,Int}(v => nextstamp() for v in keys(t)), collect(itn.ortho_region(ψ)))
end
Base.getindex(ψ::DeviceTTN, v) = ψ.t[v]
function Base.setindex!(ψ::DeviceTTN, T::DT, v)
  ψ.t[v] = T
  ψ.stamp[v] = nextstamp()
  return ψ
end
Base.copy(ψ::DeviceTTN) = DeviceTTN(ψ.ctx, ψ.graph, copy(ψ.t), copy(ψ.stamp), copy(ψ.ortho_region))
neighbors(ψ::DeviceTTN, v) = itn.neighbors(ψ.graph, v)
linkind(ψ::DeviceTTN, u, v) = only(intersect(ψ[u].inds, ψ[v].inds))
maxlinkdim(ψ::DeviceTTN) = maximum(dim(linkind(ψ, itn.src(e), itn.dst(e))) for e in itn.edges(ψ.graph); init=1)
function to_itensornetwork(ψ::DeviceTTN)
  out = itn.ITensorNetwork(ψ.graph)
  for v in keys(ψ.t)
    out[v] = download(ψ[v])
  end
  return itn.TreeTensorNetwork(out; ortho_region=ψ.ortho_region)
end

mutable struct DeviceProjTTN
  ctx::Ctx
  graph::Any
  H::Dict{Any,DT}
  envs::Dict{Any,Tuple{DT,Int}}       # directed edge (u => v) => (environment, stamp)
  pos::Vector{Any}
  psi::Union{Nothing,DeviceTTN}
end
function DeviceProjTTN(c::Ctx, H)
  H = ns.permute_indices(H)
  g = itn.underlying_graph(H)
  return DeviceProjTTN(c, g, Dict{Any,DT}(v => upload(c, H[v]) for v in itn.vertices(H)),
                       Dict{Any,Tuple{DT,Int}}(), collect(itn.vertices(H)), nothing)
end
# vertices on u's side of the edge u => v
function side(P::DeviceProjTTN, u, v)
  seen, todo = Set([v]), [u]
  out = Any[]
  while !isempty(todo)
    x = pop!(todo)
    x in seen && continue
    push!(seen, x); push!(out, x)
    append!(todo, itn.neighbors(P.graph, x))
  end
  return out
end
# environment of the directed edge u => v (the subtree on u's side), recomputed when a
# tensor on that side is newer than it (the ProjTTN cache of itn.position)
function environment(P::DeviceProjTTN, ψ::DeviceTTN, u, v)
  key = u => v
  if haskey(P.envs, key)
    E, st = P.envs[key]
    all(ψ.stamp[x] <= st for x in side(P, u, v)) && return E
  end
  inc = [environment(P, ψ, w, u) for w in itn.neighbors(P.graph, u) if w != v]
  A = ψ[u]
  # the bra: the same storage with every index primed (links and site), conjugated below
  bra = DT(A.ctx, A.h, [prime(i) for i in A.inds], A.cplx)
  E = contract(P.ctx, [A, inc..., P.H[u], bra]; conj=[false, fill(false, length(inc))..., false, true])
  P.envs[key] = (E, nextstamp())
  return E
end
incident_edges(P::DeviceProjTTN, region) =
  [(u => v) for v in region for u in itn.neighbors(P.graph, v) if !(u in region)]
function map_tensors(P::DeviceProjTTN)
  envs = [environment(P, P.psi, e.first, e.second) for e in incident_edges(P, P.pos)]
  return [envs..., (P.H[v] for v in P.pos)...]
end
position!(P::DeviceProjTTN, ψ::DeviceTTN, region) = (P.pos = collect(region); P.psi = ψ; P)

# ---------------------------------------------------------------------------
# factorizations and local solvers
# ---------------------------------------------------------------------------

function factorize(T::DT, left::Vector; cutoff=0.0, maxdim=typemax(Int), mindim=1, complement=false)
  c = T.ctx
  la = Cint[findfirst(==(i), T.inds) - 1 for i in left]
  U = Ref{Ptr{Cvoid}}(C_NULL); Cm = Ref{Ptr{Cvoid}}(C_NULL); P = Ref{Ptr{Cvoid}}(C_NULL)
  k = Ref{Int64}(); err = Ref{Float64}()
  md = Int64(min(maxdim, typemax(Int64)))
  if complement
    check(c, @ccall lib.nsg_factorize_complement(c.h::Ptr{Cvoid}, T.h::Ptr{Cvoid}, la::Ptr{Cint}, length(la)::Cint,
                                                 cutoff::Float64, md::Int64, Int64(mindim)::Int64,
                                                 U::Ptr{Ptr{Cvoid}}, Cm::Ptr{Ptr{Cvoid}}, P::Ptr{Ptr{Cvoid}},
                                                 k::Ptr{Int64}, err::Ptr{Float64})::Cint)
  else
    check(c, @ccall lib.nsg_factorize(c.h::Ptr{Cvoid}, T.h::Ptr{Cvoid}, la::Ptr{Cint}, length(la)::Cint,
                                      cutoff::Float64, md::Int64, Int64(mindim)::Int64, U::Ptr{Ptr{Cvoid}},
                                      Cm::Ptr{Ptr{Cvoid}}, k::Ptr{Int64}, err::Ptr{Float64}, C_NULL::Ptr{Float64},
                                      0::Int64)::Cint)
  end
  right = [i for i in T.inds if !(i in left)]
  l = Index(Int(k[]), "Link")
  Ut = wrap(c, U[], [left..., l], T.cplx)
  Ct = wrap(c, Cm[], [l, right...], T.cplx)
  Pt = (complement && P[] != C_NULL) ? wrap(c, P[], [left..., Index(prod(dim.(left)) - Int(k[]), "Comp")], T.cplx) :
       nothing
  return Ut, Ct, Pt, err[]
end
function qr(T::DT, left::Vector)
  c = T.ctx
  la = Cint[findfirst(==(i), T.inds) - 1 for i in left]
  Q = Ref{Ptr{Cvoid}}(C_NULL); R = Ref{Ptr{Cvoid}}(C_NULL)
  check(c, @ccall lib.nsg_qr(c.h::Ptr{Cvoid}, T.h::Ptr{Cvoid}, la::Ptr{Cint}, length(la)::Cint,
                             Q::Ptr{Ptr{Cvoid}}, R::Ptr{Ptr{Cvoid}})::Cint)
  right = [i for i in T.inds if !(i in left)]
  q = Index(min(prod(dim.(left)), prod(dim.(right))), "Link,qr")
  return wrap(c, Q[], [left..., q], T.cplx), wrap(c, R[], [q, right...], T.cplx)
end
function eigh(rho::DT, rows::Vector; cutoff=0.0, maxdim=typemax(Int), mindim=1)
  c = rho.ctx
  ra = Cint[findfirst(==(i), rho.inds) - 1 for i in rows]
  U = Ref{Ptr{Cvoid}}(C_NULL); k = Ref{Int64}(); err = Ref{Float64}()
  ev = zeros(Float64, prod(dim.(rows)))
  check(c, @ccall lib.nsg_eigh(c.h::Ptr{Cvoid}, rho.h::Ptr{Cvoid}, ra::Ptr{Cint}, length(ra)::Cint, cutoff::Float64,
                               Int64(min(maxdim, typemax(Int64)))::Int64, Int64(mindim)::Int64, U::Ptr{Ptr{Cvoid}},
                               ev::Ptr{Float64}, length(ev)::Int64, k::Ptr{Int64}, err::Ptr{Float64})::Cint)
  cols = [i for i in rho.inds if !(i in rows)]
  return wrap(c, U[], [cols..., Index(Int(k[]), "Link,exp")], rho.cplx), ev[1:k[]]
end

# eigsolve_solver (local_solvers/eigsolve.jl:3-29): Lanczos on the device
function eigsolve_solver(m::LinMap, x::DT; krylovdim=3, maxiter=1, tol=1e-14, kws...)
  λ = Ref{Float64}(); n = Ref{Cint}()
  check(m.ctx, @ccall lib.nsg_eigsolve(m.ctx.h::Ptr{Cvoid}, m.h::Ptr{Cvoid}, x.h::Ptr{Cvoid}, krylovdim::Cint,
                                       maxiter::Cint, tol::Float64, λ::Ptr{Float64}, n::Ptr{Cint})::Cint)
  return λ[], x
end
# exponentiate_solver (local_solvers/exponentiate.jl:3-29)
function exponentiate_solver(m::LinMap, t::Number, x::DT; krylovdim=30, maxiter=100, tol=1e-12, kws...)
  conv = Ref{Cint}(); n = Ref{Cint}()
  check(m.ctx, @ccall lib.nsg_exponentiate(m.ctx.h::Ptr{Cvoid}, m.h::Ptr{Cvoid}, real(t)::Float64, imag(t)::Float64,
                                           x.h::Ptr{Cvoid}, krylovdim::Cint, maxiter::Cint, tol::Float64,
                                           conv::Ptr{Cint}, n::Ptr{Cint})::Cint)
  return x, (; converged=conv[], numops=n[])
end
# runge_kutta_solver (local_solvers/runge_kutta.jl:16-25)
function runge_kutta_solver(m::LinMap, t::Number, x::DT; order=4, kws...)
  check(m.ctx, @ccall lib.nsg_runge_kutta(m.ctx.h::Ptr{Cvoid}, m.h::Ptr{Cvoid}, real(t)::Float64, imag(t)::Float64,
                                          x.h::Ptr{Cvoid}, order::Cint)::Cint)
  return x, nothing
end

# ---------------------------------------------------------------------------
# the plugins (same signatures and keyword handling as the reference)
# ---------------------------------------------------------------------------

const DevEig = ns.EigsolveProblem{<:DeviceTTN,<:DeviceProjTTN}
const DevExp = ns.ApplyExpProblem{<:DeviceTTN}

# itn.orthogonalize(ψ, region): QR walk from the current orthogonality region
function orthogonalize(ψ::DeviceTTN, region)
  path = itn.edge_sequence_between_regions(ψ.graph, ψ.ortho_region, collect(region))
  ψ = copy(ψ)
  for e in path
    s, d = itn.src(e), itn.dst(e)
    left = [i for i in ψ[s].inds if !(i in ψ[d].inds)]
    Q, R = qr(ψ[s], left)
    ψ[s] = Q
    ψ[d] = contract(ψ.ctx, [R, ψ[d]])
  end
  ψ.ortho_region = collect(region)
  return ψ
end

# extracter.jl:3-17
function ns.extracter(problem::Union{DevEig,DevExp}, region_iterator; sweep, trunc=(;), kws...)
  return phase(ns.state(problem).ctx, :extract) do
    trunc = ns.truncation_parameters(sweep; trunc...)
    region = ns.current_region(region_iterator)
    psi = orthogonalize(ns.state(problem), region)
    local_state = length(region) == 1 ? psi[only(region)] : contract(psi.ctx, [psi[v] for v in region])
    problem = setproperties(problem; state=psi)
    problem, local_state = ns.subspace_expand(problem, local_state, region_iterator; sweep, trunc, kws...)
    P = ns.operator(problem)
    position!(P, ns.state(problem), region)
    return setproperties(problem; operator=P), local_state
  end
end

# subspace/densitymatrix.jl:5-74 on the device
function ns.subspace_expand(::ns.Backend"densitymatrix", problem::Union{DevEig,DevExp}, local_state::DT,
                            region_iterator; north_pass=1, expansion_factor=ns.default_expansion_factor(),
                            max_expand=ns.default_max_expand(), trunc, kws...)
  return phase(ns.state(problem).ctx, :subspace) do
  region = ns.current_region(region_iterator)
  psi = copy(ns.state(problem))
  P = ns.operator(problem)
  prev = setdiff(P.pos, region)
  length(prev) != 1 && return problem, local_state
  pv = only(prev)
  A = psi[pv]
  nxt = filter(v -> !isempty(intersect(psi[v].inds, A.inds)), region)
  isempty(nxt) && return problem, local_state
  nv = only(nxt)
  C = psi[nv]
  a = only(intersect(A.inds, C.inds))
  basis = prod(dim(i) for i in A.inds if !(i in C.inds))
  expand = ns.compute_expansion(dim(a), basis; expansion_factor, max_expand, maxdim=trunc.maxdim)
  expand <= 0 && return problem, local_state
  envs = [environment(P, psi, e.first, e.second) for e in incident_edges(P, P.pos)
          if !(e.first in region || e.second in region)]
  sqrt_rho = contract(psi.ctx, [A, envs..., P.H[pv]])
  # the complement projections, rho and its truncated eigenvectors, the orthogonality
  # guard and the direct sum, as in the reference; every step on the device
  ket = [i for i in A.inds if i != a]
  for _ in 1:north_pass
    Ap = DT(A.ctx, A.h, [prime(i) for i in A.inds], A.cplx)
    proj = contract(psi.ctx, [Ap, contract(psi.ctx, [Ap, sqrt_rho]; conj=[true, false])])
    check(psi.ctx, @ccall lib.nsg_axpby(psi.ctx.h::Ptr{Cvoid}, -1.0::Float64, 0.0::Float64, proj.h::Ptr{Cvoid},
                                        1.0::Float64, 0.0::Float64, sqrt_rho.h::Ptr{Cvoid})::Cint)
  end
  snp = DT(sqrt_rho.ctx, sqrt_rho.h, [noprime(i) for i in sqrt_rho.inds], sqrt_rho.cplx)
  rho = contract(psi.ctx, [sqrt_rho, snp]; conj=[false, true])
  U, _ = eigh(rho, [prime(i) for i in ket]; trunc..., maxdim=expand)
  guard = contract(psi.ctx, [U, A]; conj=[true, false])
  norm(guard) > 1e-10 && return problem, local_state
  u = last(U.inds)
  r = Ref{Ptr{Cvoid}}(C_NULL)
  Up = permute(U, [ket..., u])
  check(psi.ctx, @ccall lib.nsg_concat(psi.ctx.h::Ptr{Cvoid}, permute(A, [ket..., a]).h::Ptr{Cvoid}, Up.h::Ptr{Cvoid},
                                       length(ket)::Cint, r::Ptr{Ptr{Cvoid}})::Cint)
  ax = Index(dim(a) + dim(u), "Link")
  Ax = wrap(psi.ctx, r[], [ket..., ax], A.cplx)
  expander = contract(psi.ctx, [Ax, A]; conj=[true, false])
  psi[pv] = Ax
  psi[nv] = contract(psi.ctx, [expander, C])
  local_state = contract(psi.ctx, [expander, local_state])
  return setproperties(problem; state=psi), local_state
  end  # phase
end

# eigsolve.jl:14-28
function ns.updater(E::DevEig, local_state::DT, region_iterator; outputlevel, solver=eigsolve_solver, kws...)
  P = ns.operator(E)
  return phase(P.ctx, :krylov) do
    m = LinMap(P.ctx, map_tensors(P), local_state.inds)
    eigval, x = solver(m, local_state; kws...)
    return setproperties(E; eigenvalue=eigval), x
  end
end

# applyexp.jl:18-48 (the 1-site bond back-evolution included)
function ns.updater(T::DevExp, local_state::DT, region_iterator; nsites, time_step, solver=runge_kutta_solver,
                    outputlevel, kws...)
  P = ns.operator(T)
  local_state = phase(P.ctx, :krylov) do
    first(solver(LinMap(P.ctx, map_tensors(P), local_state.inds), time_step, local_state; kws...))
  end
  if nsites == 1
    curr, nxt = ns.current_region(region_iterator), ns.next_region(region_iterator)
    if !isnothing(nxt) && nxt != curr
      e = first(itn.edge_sequence_between_regions(ns.state(T).graph, curr, nxt))
      v1, v2 = itn.src(e), itn.dst(e)
      psi = copy(ns.state(T))
      left = [i for i in local_state.inds if !(i in psi[v2].inds)]
      Q, R = qr(local_state, left)
      psi[v1] = Q
      envs = [environment(P, psi, v1, v2), environment(P, psi, v2, v1)]
      Rt, _ = solver(LinMap(P.ctx, envs, R.inds), -time_step, R; kws...)
      local_state = contract(psi.ctx, [psi[v1], Rt])
    end
  end
  return setproperties(T; current_time=ns.current_time(T) + time_step), local_state
end

# inserter.jl:3-33
function ns.inserter(problem::Union{DevEig,DevExp}, local_tensor::DT, region_iterator; normalize=false,
                     set_orthogonal_region=true, sweep, trunc=(;), kws...)
  return phase(ns.state(problem).ctx, :factorize) do
  trunc = ns.truncation_parameters(sweep; trunc...)
  region = ns.current_region(region_iterator)
  psi = copy(ns.state(problem))
  if length(region) == 1
    C = local_tensor
  elseif length(region) == 2
    U, C, _, _ = factorize(local_tensor, [i for i in psi[first(region)].inds if i in local_tensor.inds]; trunc...)
    psi[first(region)] = U
  else
    error("Region of length $(length(region)) not currently supported")
  end
  v = last(region)
  psi[v] = C
  set_orthogonal_region && (psi.ortho_region = [v])
  normalize && scale!(psi[v], 1 / norm(psi[v]))
  return setproperties(problem; state=psi)
  end  # phase
end

ns.state(ψ::DeviceTTN) = ψ
itn.maxlinkdim(ψ::DeviceTTN) = maxlinkdim(ψ)

# ---------------------------------------------------------------------------
# one fused call per chain region (nsg_region_step), for chain drivers that hand the
# whole two-site step to the device
# ---------------------------------------------------------------------------

function region_step(c::Ctx, L::DT, W1::DT, W2::DT, R::DT, psi1::DT, psi2::DT; direction=0, krylovdim=3,
                     maxiter=1, tol=1e-14, cutoff=0.0, maxdim=typemax(Int), mindim=1)
  U = Ref{Ptr{Cvoid}}(C_NULL); Cm = Ref{Ptr{Cvoid}}(C_NULL); E = Ref{Float64}(); k = Ref{Int64}()
  err = Ref{Float64}()
  check(c, @ccall lib.nsg_region_step(c.h::Ptr{Cvoid}, L.h::Ptr{Cvoid}, W1.h::Ptr{Cvoid}, W2.h::Ptr{Cvoid},
                                      R.h::Ptr{Cvoid}, psi1.h::Ptr{Cvoid}, psi2.h::Ptr{Cvoid}, direction::Cint,
                                      krylovdim::Cint, maxiter::Cint, tol::Float64, cutoff::Float64,
                                      Int64(min(maxdim, typemax(Int64)))::Int64, Int64(mindim)::Int64,
                                      U::Ptr{Ptr{Cvoid}}, Cm::Ptr{Ptr{Cvoid}}, E::Ptr{Float64}, k::Ptr{Int64},
                                      err::Ptr{Float64})::Cint)
  return E[], U[], Cm[], k[], err[]
end

# the timeout path of the bounded device waits (returns the status, does not throw)
wait_probe(c::Ctx, polls::Integer) = @ccall lib.nsg_ctx_wait_probe(c.h::Ptr{Cvoid}, Int64(polls)::Int64)::Cint

end # module
