"""Single-kernel timings of the sweep's hot operations on the library stream.

    python kernelbench.py factorize --n 1024 [--complex] [--precision fp64]
    python kernelbench.py heff --chi 512 [--precision ozaki]
    python kernelbench.py gemm --m 4096 --n 4096 --k 4096 [--precision ozaki]
    python kernelbench.py region --chi 1024 --chi-right 512 [--precision ozaki]

`factorize` is the inserter's truncated factorization (it.factorize, inserter.jl:23) of
an n x n two-site matrix keeping n/2 states; `heff` one application of the two-site
chain H_eff (optimal_map, operator_map.jl:3-10) at bond dimension chi with the
Heisenberg MPO (w = 5, d = 2); `gemm` one plain product; `region` one full two-site
DMRG region step (extracter with density-matrix expansion, Lanczos updater, inserter;
iterators.jl:81-100) in the middle of a 24-site Heisenberg chain whose bonds are --chi
left of the region and --chi-right from it on (the shape of a left-to-right sweep that
raises the bond dimension from chi-right to chi), maxdim --maxdim (default --chi; with
--chi 475 --chi-right 475 --maxdim 1024 the shape of the converged N=100 sweep, where
the expansion doubles the bond before the truncation brings it back).  For `region` the
--warmup calls step the regions before the timed ones, so every timed call is the next
region of the same sweep.  Each runs --warmup untimed
and --reps timed calls and prints one JSON line with the mean time per call (CUDA
events on the library's stream) and, with --profile, the per-class kernel times.
These are small, self-contained cases meant for profiler captures of one kernel.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

from networksolvers_gb300 import _native  # noqa: E402
from networksolvers_gb300.itensors import DTensor, Index, contract, factorize  # noqa: E402
from networksolvers_gb300.network import LinearMap  # noqa: E402


class _FixedMap:
    """The four fixed tensors of a two-site chain region, in ProjTTN.map_tensors order."""

    def __init__(self, tensors):
        self.tensors = tensors

    def map_tensors(self):
        return self.tensors


def _heff_case(chi, seed):
    from networksolvers_gb300.models import heisenberg_chain
    rng = np.random.default_rng(seed)
    W = heisenberg_chain(4).tensors[2]  # bulk MPO tensor [left, s', s, right]
    w, d = W.shape[0], W.shape[1]
    a, b, s1, s2 = Index(chi), Index(chi), Index(d), Index(d)
    w1, w2, w3 = Index(w), Index(w), Index(w)
    L = rng.standard_normal((chi, w, chi))
    R = rng.standard_normal((chi, w, chi))
    fixed = [DTensor.from_numpy(L + L.transpose(2, 1, 0), [a.prime(), w1, a]),
             DTensor.from_numpy(R + R.transpose(2, 1, 0), [b.prime(), w3, b]),
             DTensor.from_numpy(W, [w1, s1.prime(), s1, w2]),
             DTensor.from_numpy(W, [w2, s2.prime(), s2, w3])]
    inds = [a, s1, s2, b]
    x = DTensor.from_numpy(rng.standard_normal((chi, d, d, chi)), inds)
    return LinearMap(_FixedMap(fixed), inds), x


def _region_case(chi, chi_right, precision, seed, ctx, maxdim=None):
    from networksolvers_gb300 import models
    from networksolvers_gb300.network import euler_sweep
    from networksolvers_gb300.sweep import EigsolveProblem, RegionIterator, _prepare, region_iterator_action, updater_eigsolve
    nsites = 24
    g = models.chain_graph(nsites)
    mid = nsites // 2
    psi0 = models.random_state(g, 1, seed=seed)
    rng = np.random.default_rng(seed)
    dims = {}
    for (u, v) in g.edges:
        i = min(u, v)
        cap = 2 ** min(i, nsites - i)
        dims[(u, v)] = min(cap, chi if i < mid else chi_right)
    for v in g.vertices:
        shape = [2 if leg[0] == 's' else dims[leg[1]] for leg in psi0.legs[v]]
        psi0.tensors[v] = rng.standard_normal(shape) / np.sqrt(np.prod(shape))
    H = models.heisenberg_chain(nsites)
    psi, P = _prepare(H, psi0, ctx)
    prob = EigsolveProblem(psi, P)
    trunc = dict(cutoff=1e-12, maxdim=maxdim or chi)
    plan = euler_sweep(psi.g, 2)
    R = RegionIterator(prob, plan)
    first = [k for k, (region, _) in enumerate(plan) if region[0] == mid][0]
    kws = dict(extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
               updater_kwargs=dict(krylovdim=3, maxiter=1), inserter_kwargs=dict(trunc=trunc))
    state = {"prob": prob, "k": first - 1}

    def step():
        state["k"] += 1
        R.which = state["k"]
        state["prob"] = region_iterator_action(state["prob"], R, updater_eigsolve, sweep=1, **kws)

    return step


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python kernelbench.py")
    ap.add_argument("op", choices=["factorize", "heff", "gemm", "region"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--m", type=int, default=4096)
    ap.add_argument("--k", type=int, default=4096)
    ap.add_argument("--chi", type=int, default=512)
    ap.add_argument("--chi-right", type=int, default=None)
    ap.add_argument("--maxdim", type=int, default=None,
                    help="region: truncation maxdim (default --chi); above --chi the densitymatrix expansion "
                         "enlarges the bond as in a converged sweep of a larger maxdim")
    ap.add_argument("--complex", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=sorted(_native.PRECISIONS))
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--profile", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)

    ctx = _native.Context(0, precision=args.precision)
    _native.set_default_context(ctx)
    rng = np.random.default_rng(args.seed)
    flops = None
    if args.op == "factorize":
        n = args.n
        M = rng.standard_normal((n, n))
        if args.complex:
            M = M + 1j * rng.standard_normal((n, n))
        l, r = Index(n), Index(n)
        T = DTensor.from_numpy(M, [l, r])
        run = lambda: factorize(T, [l], cutoff=1e-12, maxdim=n // 2)
        case = {"n": n, "keep": n // 2, "complex": args.complex}
    elif args.op == "heff":
        lm, x = _heff_case(args.chi, args.seed)
        run = lambda: lm(x)
        flops = lm.flops()
        case = {"chi": args.chi, "w": 5, "d": 2}
    elif args.op == "region":
        run = _region_case(args.chi, args.chi_right or args.chi // 2, args.precision, args.seed, ctx, args.maxdim)
        case = {"chi": args.chi, "chi_right": args.chi_right or args.chi // 2, "sites": 24,
                "maxdim": args.maxdim or args.chi}
    else:
        i, j, l = Index(args.m), Index(args.n), Index(args.k)
        A = DTensor.from_numpy(rng.standard_normal((args.m, args.k)), [i, l])
        B = DTensor.from_numpy(rng.standard_normal((args.k, args.n)), [l, j])
        run = lambda: contract([A, B], out=[i, j])
        flops = 2.0 * args.m * args.n * args.k
        case = {"m": args.m, "n": args.n, "k": args.k}
    for _ in range(args.warmup):
        run()
    ctx.synchronize()
    if args.profile:
        ctx.profile(True)
    launches0 = ctx.counters()["launches"]
    ctx.record(0)
    for _ in range(args.reps):
        run()
    ctx.record(1)
    ms = ctx.elapsed_ms(0, 1) / args.reps
    line = {"op": args.op, "case": case, "precision": args.precision, "reps": args.reps, "ms_per_call": ms,
            "launches_before_timed": int(launches0),
            "launches_per_call": (ctx.counters()["launches"] - launches0) / args.reps}
    if flops:
        line["tflops_fp64_equiv"] = flops / (ms / 1e3) / 1e12
    if args.profile:
        line["classes_ms_per_call"] = {k: v["ms"] / args.reps for k, v in ctx.profile_read().items()
                                       if v["launches"]}
        ctx.profile(False)
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
