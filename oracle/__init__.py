"""FP64 CPU restatement of NetworkSolvers.jl's sweep hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this package; only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it,
and only as the checker / the timed CPU path, never as the thing measured on GPU.

What it restates (reference = emstoudenmire/NetworkSolvers.jl, paths relative to
that project):

* driver: iterators.jl:81-100 (extract → update → insert), sweep_solve.jl:12-40
* region plans: region_plans/euler_tour.jl:13-48, euler_plans.jl:4-13,
  dfs_plans.jl:5-22, tdvp_region_plans.jl:1-44
* plugins: extracter.jl:3-17, inserter.jl:3-33, eigsolve.jl:14-28,
  applyexp.jl:18-48, subspace/subspace.jl:8-48, subspace/densitymatrix.jl:5-74,
  truncation_parameters.jl:1-14, operator_map.jl:3-10
* local solvers: local_solvers/eigsolve.jl:3-29, exponentiate.jl:3-29,
  runge_kutta.jl:2-25
* un-vendored dependencies, restated from their documented behaviour (not copied):
  ITensors/NDTensors truncated SVD (`factorize`, relative discarded-weight cutoff
  on σ², maxdim, mindim), Hermitian `eigen` with the same truncation, `qr`,
  `directsum`; KrylovKit Lanczos `eigsolve` and `exponentiate`;
  ITensorNetworks `orthogonalize`, `ProjTTN`/`position`/`environment`.

Parity status: the restatement is pinned against exact diagonalisation
(`oracle.ed`, scipy) on the reference's own test graphs and assertions
(test/dmrg/test_tree_dmrg.jl:53,67; test/tdvp/test_tree_tdvp.jl:65-77;
test/test_euler_tour.jl:13-25).  Bit-level parity with the Julia stack
(ITensors/KrylovKit) is unpinned: no Julia is available to run the reference.
"""
