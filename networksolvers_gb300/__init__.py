"""GB300-native sweep kernels for NetworkSolvers.jl (DMRG / TDVP region steps).

Public API (same names as NetworkSolvers.jl): `dmrg`/`eigsolve`, `tdvp`/`applyexp`,
the plugins `extracter`, `updater_eigsolve`, `updater_applyexp`, `inserter`,
`subspace_expand`, the local solvers `eigsolve_solver`, `exponentiate_solver`,
`runge_kutta_solver`, the region plans, the fused chain `region_step`, `OpSum` /
`chain_mpo` / `ttn_operator` for Hamiltonians on chains and trees, `batch.SolvePool` for many concurrent solves, and the
U(1) block-sparse layer `qn` (`qn_dmrg_chain`, block tensors) for conserve_qns runs.  The
numerics run in libnsg.so (include/nsg.h); `build_library()` compiles it for sm_103a.
"""
from . import models
from .build import build as build_library
from .sweep import (dmrg, eigsolve, tdvp, applyexp, extracter, inserter, subspace_expand,
                    updater_eigsolve, updater_applyexp, eigsolve_solver, exponentiate_solver,
                    runge_kutta_solver, truncation_parameters, sweep_solve, region_iterator_action,
                    region_step, EigsolveProblem, ApplyExpProblem)
from .network import (euler_tour_edges, euler_tour_vertices, euler_sweep, post_order_dfs_plan,
                      tdvp_regions, tdvp_sub_time_steps, TTN, ProjTTN, LinearMap, inner)
from ._native import Context, default_context, set_default_context, set_thread_context, NsgError
from .models import OpSum, chain_mpo, ttn_operator
from . import qn
from .qn import qn_dmrg_chain

__all__ = [n for n in dir() if not n.startswith("_")]
