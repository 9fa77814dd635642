"""Benchmark: 2-site DMRG sweeps on the N=100 Heisenberg chain on one GB300.

Workload (the "large 2-site DMRG" configuration): S=1/2 Heisenberg chain N=100, J=1,
open boundaries, MPO bond dimension 5; random MPS at bond dimension 32 from seed 1
(own PCG64 generator); maxdim schedule [64, 128, 256, 512, 1024] by sweep, cutoff
1e-12, densitymatrix subspace expansion on, Lanczos krylovdim 3 / maxiter 1.
One step = one full sweep (198 two-site regions).  Warm-up steps are the first W sweeps
of the schedule, the timed steps the next K sweeps.  Metric: sweeps/s (higher is
better); the split-precision form is the product path: the large contractions (H_eff,
environments) run as six-slice BF16 products with exact FP32 chunk accumulation on
tcgen05, the factorization's Gram matrices, the eigensolver's GEMMs, `C = U^H M` and the
density-matrix expansion as eight-slice products (FP64 accuracy), while the
tridiagonalisation, the secular equations and the Lanczos scalars stay FP64;
`--precision tf32x3` is the three-product TF32 form and `--precision fp64` the plain form
(every contraction on the FP64 CUDA cores).  Other workloads
(`--workload c1|tdvp|batch|serve|accuracy|qn`) print their own lines; see `main()`.

Timing: CUDA events on the library's stream around each timed sweep; the per-kernel
roofline and the kernel shares come from events around each launch of the kernel
classes in one further sweep after the timed ones (nothing is recorded inside the timed
sweeps).  Inputs larger than L2: the two-site tensors, environments and GEMM
operands at bond dimension >= 512 are 8-170 MB each and are rewritten every region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SITES, CHI0, SEED = 100, 32, 1
SCHEDULE = [64, 128, 256, 512, 1024]
CUTOFF = 1e-12
REGIONS_PER_SWEEP = 2 * (N_SITES - 1)


# GB300 FP64 rate: the measured peaks hold no FP64 figure; kernelbench's FP64 GEMM at
# 4096^3 reaches 1.25 TFLOP/s (cuBLAS DGEMM 1.10) on these GPUs, the nominal figure
FP64_PEAK_TFLOPS = 1.25
FP64_PEAK_NOTE = "GB300 FP64 rate (no FP64 figure in the measured peaks; 1.25 TFLOP/s nominal)"


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.rows, self.proc = [], None

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace('.', '', 1).isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def replica_time(t_local, device=None):
    """Slowest replica's time: MAX all-reduce over the process group when one is
    initialised (the replicas share no data; only this scalar crosses ranks)."""
    import torch.distributed as td
    if not (td.is_available() and td.is_initialized()):
        return t_local
    import torch
    tt = torch.tensor([t_local], dtype=torch.float64, device=device or "cpu")
    td.all_reduce(tt, op=td.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(world, steps, t_max):
    """Whole-job throughput of `world` replicas that each ran `steps` steps."""
    return world * steps / t_max


def workload():
    import networksolvers_gb300.models as m
    return m.heisenberg_chain(N_SITES), m.random_state(m.chain_graph(N_SITES), CHI0, seed=SEED)


def kwargs_for(sweep_offset=0):
    sched = SCHEDULE[sweep_offset:] if sweep_offset < len(SCHEDULE) else [SCHEDULE[-1]]
    trunc = dict(cutoff=CUTOFF, maxdim=sched)
    return dict(nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
                extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
                inserter_kwargs=dict(trunc=trunc))


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (the reference's sweep restated on FP64 numpy/OpenBLAS)
# running real region steps of the workload's sweep, one region per step
# ---------------------------------------------------------------------------

# Largest bond dimension of each sweep of this workload's 10-sweep schedule and beyond,
# as the split-precision GPU run reaches them (the bond dimension saturates near 475 once
# the cutoff 1e-12 governs the truncation); the reference arm samples region steps at
# these sizes, the GPU arm passes the sizes it actually reached.
SWEEP_BOND = {1: 64, 2: 128, 3: 256, 4: 512, 5: 1024, 6: 1024, 7: 1024, 8: 1024, 9: 863, 10: 600}
CONVERGED_BOND = 475


def sweep_bond(sweep):
    return SWEEP_BOND.get(sweep, CONVERGED_BOND)


def cpu_region_step(sweep, position, cap, seed):
    """Seconds the oracle takes for region `position` (0..197) of sweep `sweep` of the
    workload: the complete reference region step (extracter with the densitymatrix
    expansion, Lanczos with 3 H_eff applications, truncated factorization; iterators.jl:
    81-100) on all host threads.  The state is a seeded random MPS in the gauge the sweep
    has at that region (orthogonality centre on the region's first vertex) with bond
    dimensions min(2^i, 2^(N-i), cap), on the window of the chain the step reads: the
    region, the previous region's vertex and enough sites on either side (an open
    Heisenberg block) for the bonds to reach `cap`.  Building the state, its gauge and
    the cached environments is not timed; the step itself is."""
    import math
    from oracle import sweep as osw
    from oracle.network import G, ProjTTN, euler_sweep, from_network, orthogonalize
    import networksolvers_gb300.models as m
    cg = m.chain_graph(N_SITES)
    plan = euler_sweep(G(cg.vertices, cg.edges), 2)
    region = list(plan[position][0])
    prev = list(plan[position - 1][0]) if position > 0 else list(plan[-1][0])
    lb = int(math.ceil(math.log2(cap))) + 1
    lo = max(1, min(region + prev) - lb)
    hi = min(N_SITES, max(region + prev) + lb)
    nw = hi - lo + 1
    g = m.chain_graph(nw)
    sub = lambda v: v - lo + 1
    H = m.heisenberg_chain(nw)
    rng = np.random.Generator(np.random.PCG64(seed))
    tensors, legs = {}, {}
    for v in g.vertices:
        lg = m._permuted_legs(g, v, 'l', [('s', v)])
        shape = []
        for leg in lg:
            if leg[0] == 's':
                shape.append(2)
            else:
                i = min(leg[1])  # bond between sub-chain sites i and i+1
                ir = lo - 1 + i  # the same bond of the full chain
                shape.append(int(min(cap, 2 ** min(i, nw - i, 30), 2 ** min(ir, N_SITES - ir, 30))))
        tensors[v] = rng.standard_normal(shape)
        legs[v] = lg
    net = m.Network(g, tensors, legs, np.float64, {"kind": "state", "ortho_region": list(g.vertices)})
    psi, sites = from_network(net)
    (_, Ht), _ = from_network(H, site_index=sites)
    a, b = sub(region[0]), sub(region[1])
    pr = [sub(v) for v in prev]
    psi = orthogonalize(psi, [a])
    psi[a] = psi[a] / psi[a].norm()
    P = ProjTTN(psi.g, Ht)
    # environments the step reads from the cache: everything outside the region and the
    # previous region's vertex
    pv = [v for v in pr if v not in (a, b)]
    for (u, v) in P.incident_edges(pr + [a, b]):
        P.environment(psi, u, v)
    P.position(psi, pr)
    prob = osw.EigsolveProblem(psi, P)
    kw = kwargs_for(0)
    rkw = dict(extracter_kwargs=kw["extracter_kwargs"], updater_kwargs=kw["updater_kwargs"],
               inserter_kwargs=kw["inserter_kwargs"], outputlevel=0)
    R = osw.RegionIterator(prob, [(pr, rkw), ([a, b], rkw)])
    R.which = 1
    t = time.perf_counter()
    osw.region_iterator_action(prob, R, osw.updater_eigsolve, sweep=sweep, **rkw)
    return time.perf_counter() - t, (pv, len(pr))


def cpu_sweep_sample(sweeps, caps, seed=11):
    """One oracle region step per sweep in `sweeps` (largest bond `caps[k]`), at region
    positions spread evenly over the sweep (stratified: step k runs region
    floor((k + 1/2) 198 / len(sweeps))).  Returns the per-step seconds."""
    out = []
    n = len(sweeps)
    for k, (sw, cap) in enumerate(zip(sweeps, caps)):
        pos = int((k + 0.5) * REGIONS_PER_SWEEP / n)
        t, _ = cpu_region_step(sw, pos, cap, seed + k)
        out.append(t)
    return out


def run_reference(args):
    """CPU reference arm: the oracle (FP64 numpy/OpenBLAS on all host threads) running
    region steps of the workload's sweeps W+1..W+K, one region per step (W warm-up steps
    before them); sweeps/s = regions run / 198 / their measured time."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    warm = list(range(1, args.warmup + 1))
    timed = list(range(args.warmup + 1, args.warmup + args.steps + 1))
    cpu_sweep_sample(warm, [sweep_bond(s) for s in warm], seed=5)
    steps = cpu_sweep_sample(timed, [sweep_bond(s) for s in timed])
    t = float(np.sum(steps))
    v = args.steps / REGIONS_PER_SWEEP / t
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": "dmrg_sweeps_per_s", "value": v, "unit": "sweeps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(1),
            "cpu_baseline": {"value": v, "unit": "sweeps/s", "cores": cores, "kind": "port",
                             "sample": f"one oracle region step per step (densitymatrix expansion, Lanczos with 3 "
                                       f"H_eff applications, truncated factorization) of sweeps {timed[0]}-{timed[-1]}"
                                       f" at region positions spread evenly over the sweep, bond dimensions "
                                       f"{sorted(set(sweep_bond(s) for s in timed))} as the sweeps reach them; "
                                       f"value = steps / 198 / measured time"},
            "step_seconds": steps,
            "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(world):
    return {"workload": "heisenberg_chain_N100_2site_dmrg_maxdim1024", "global_batch": world, "seq_len": N_SITES,
            "parallelism": f"replicas{world}"}


def run_nsg(args):
    import networksolvers_gb300 as ns
    from networksolvers_gb300 import _native
    from networksolvers_gb300.sweep import _prepare
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
    ctx = _native.Context(local, precision=args.precision)
    _native.set_default_context(ctx)
    H, psi0 = workload()
    psi, P = _prepare(H, psi0, ctx)
    kw = kwargs_for(0)
    from networksolvers_gb300.sweep import EigsolveProblem, sweep_solve, updater_eigsolve
    from networksolvers_gb300.network import euler_sweep
    prob = EigsolveProblem(psi, P)
    energies, maxdims, sweep_ms, all_ms = [], [], [], []
    plan = lambda: euler_sweep(psi.g, 2, **dict(extracter_kwargs=kw["extracter_kwargs"],
                                                 updater_kwargs=kw["updater_kwargs"],
                                                 inserter_kwargs=kw["inserter_kwargs"], outputlevel=0))
    from networksolvers_gb300.sweep import RegionIterator, region_iterator_action

    def one_sweep(sweep):
        nonlocal prob
        pl = plan()
        R = RegionIterator(prob, pl)
        for k, (region, rkws) in enumerate(pl):
            R.which = k
            prob = region_iterator_action(prob, R, updater_eigsolve, sweep=sweep, **dict(rkws))

    total = args.warmup + args.steps
    clocks = Clocks()
    launches0 = launches1 = 0
    for sweep in range(1, total + 1):
        timed = sweep > args.warmup
        if timed and sweep == args.warmup + 1:
            if rank == 0 and not args.no_e2e:
                # host copy of the state entering the timed sweeps (outside the timed region):
                # the e2e leg replays the same sweeps from it through the public API
                snap = (prob.state.to_numpy(psi0), list(prob.state.ortho_region))
            if dist:
                td.barrier()
            ctx.synchronize()
            clocks.start()
            launches0 = ctx.counters()["launches"]
        ctx.record(0)
        one_sweep(sweep)  # one sweep of the schedule (the sweep index drives get_or_last)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        all_ms.append(ms)
        energies.append(prob.eigenvalue)
        maxdims.append(prob.state.maxlinkdim())
        if timed:
            sweep_ms.append(ms)
    ctx.synchronize()
    launches1 = ctx.counters()["launches"]
    if dist:
        td.barrier()
    clk = clocks.stop()
    launches = launches1 - launches0
    t_sweep = replica_time(float(np.sum(sweep_ms)) / 1e3, device="cuda" if dist else None)
    value = replica_throughput(world, args.steps, t_sweep)
    # kernel shares and the roofline come from one further sweep with CUDA events around
    # every launch of the profiled kernel classes (outside the timed sweeps)
    ctx.profile(True)
    ctx.record(0)
    one_sweep(total + 1)
    ctx.record(1)
    prof_sweep_ms = ctx.elapsed_ms(0, 1)
    prof = ctx.profile_read()
    ctx.profile(False)
    # e2e: the timed sweeps again through the public API from host buffers, one `dmrg`
    # call per sweep (upload of the state and the operator, environments built from
    # scratch, the sweep, download of the state), from the host copy taken before them
    e2e = None
    if rank == 0 and not args.no_e2e:
        from networksolvers_gb300.models import Network
        arrays, ortho = snap
        h2d = d2h = 0
        t0 = time.perf_counter()
        for k in range(args.steps):
            # the host copy keeps the state's gauge (its orthogonality centre), as a TTN does
            host_state = Network(psi0.graph, arrays, psi0.legs, np.float64, {"kind": "state", "ortho_region": ortho})
            h2d += sum(a.nbytes for a in arrays.values()) + sum(t.nbytes for t in H.tensors.values())
            E2, psi2 = ns.dmrg(H, host_state, nsweeps=1, **kwargs_for(args.warmup + k))
            arrays, ortho = psi2.to_numpy(psi0), list(psi2.ortho_region)
            d2h += sum(a.nbytes for a in arrays.values()) + 8
        t1 = time.perf_counter()
        e2e = {"value": args.steps / (t1 - t0), "unit": "sweeps/s", "h2d_bytes_per_step": int(h2d // args.steps),
               "d2h_bytes_per_step": int(d2h // args.steps), "energy": E2}
    bf16, hbm, kind = peaks()
    # roofline of the dominant kernel class of the profiled sweep
    classes = {k: v for k, v in prof.items() if v["launches"] > 0}
    dom = max(classes, key=lambda k: classes[k]["ms"]) if classes else None
    tot_ms = sum(v["ms"] for v in classes.values())
    roof = None
    if dom == "tc_gemm":
        c = classes[dom]
        if args.precision == "ozaki":
            # 21 BF16 slice products per FP64-equivalent flop
            achieved = 21.0 * c["flops"] / (c["ms"] / 1e3) / 1e12
            peak, kname, note = bf16, "oz_gemm_kernel", f"bf16 dense ({kind})"
        else:
            achieved = 3.0 * c["flops"] / (c["ms"] / 1e3) / 1e12  # three TF32 products
            peak, kname, note = bf16 / 2.0, "tc_gemm_tf32x3_kernel", f"bf16 dense ({kind}) / 2 for kind::tf32"
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": kname, "peak_note": note}
    elif dom is not None:
        c = classes[dom]
        achieved = c["flops"] / (c["ms"] / 1e3) / 1e12
        fp64_peak = FP64_PEAK_TFLOPS
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": None, "kernel": dom,
                "peak_note": FP64_PEAK_NOTE}
        if dom == "tridiag":
            # DRAM bytes of one launch from the ncu capture at n = 950 (7.28 MB read + 1.87 MB
            # written: the L2-resident matrix once, the reflectors back), scaled by n^2 to the
            # launches' mean order, which the algorithmic flops per launch (4/3 n^3) give
            n_eff = (0.75 * c["flops"] / c["launches"]) ** (1.0 / 3.0)
            roof["traffic"] = 9.15e6 * (n_eff / 950.0) ** 2
            roof["traffic_note"] = (f"bytes per launch at the launches' mean order n = {n_eff:.0f} (from 4/3 n^3 "
                                    f"flops per launch), scaled by n^2 from ncu at n=950")
    if roof is not None:
        roof["measured_in"] = f"sweep {total + 1} (CUDA events around each launch of the class; outside the timed sweeps)"
    tc = classes.get("tc_gemm")
    heff_tflops = (tc["flops"] / (tc["ms"] / 1e3) / 1e12) if tc else None
    cpu = None
    if rank == 0 and not args.no_cpu:
        timed_sweeps = list(range(args.warmup + 1, total + 1))
        secs = cpu_sweep_sample(timed_sweeps, maxdims[args.warmup:total])
        cv = args.steps / REGIONS_PER_SWEEP / float(np.sum(secs))
        cpu = {"value": cv, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"one oracle region step per timed sweep ({args.steps} steps, {float(np.sum(secs)):.1f} s), "
                         f"region positions spread evenly over the sweep, at the largest bond dimension each timed "
                         f"sweep reached; value = steps / 198 / measured time"}
    tts = None
    if total >= 10:
        tts = {"sweeps": 10, "seconds": float(np.sum(all_ms[:10])) / 1e3, "energy": energies[9],
               "note": "the configuration's 10-sweep run (sweeps 1-10 of this run, CUDA events); timed sweeps past "
                       "sweep 10 repeat the converged state"}
    if rank == 0:
        cfg = config_dict(world)
        cfg.update({"timed_sweeps": list(range(args.warmup + 1, args.warmup + args.steps + 1)),
                    "maxdim_schedule": SCHEDULE, "precision": args.precision,
                    "l2": "operands 8-170 MB per GEMM at bond dim >= 512 (larger than L2)"})
        line = {"metric": "dmrg_sweeps_per_s", "value": value, "unit": "sweeps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_sweep * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else f"{args.precision}+f64",
                "data": "synthetic", "config": cfg,
                "energy": energies[-1], "energies_per_sweep": energies, "maxlinkdim_per_sweep": maxdims,
                "sweep_ms": sweep_ms, "all_sweep_ms": all_ms, "time_to_solution": tts,
                "heff_gemm_tflops_fp64_equiv": heff_tflops,
                "kernel_share": {k: v["ms"] / tot_ms for k, v in classes.items()} if tot_ms else {},
                "profiled_sweep_ms": prof_sweep_ms,
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "launches_before_timed": int(launches0),
                "clocks": clk}
        print(json.dumps(line), flush=True)
    if dist:
        td.destroy_process_group()


# ---------------------------------------------------------------------------
# further workloads (one JSON line each; the default is the N=100 DMRG benchmark)
# ---------------------------------------------------------------------------


def _line(**kw):
    base = {"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic"}
    base.update(kw)
    print(json.dumps(base), flush=True)


def _oracle_sweep_seconds(run, first, count):
    """CPU baseline leg: run an oracle driver with a sweep callback and return the wall
    time of sweeps first..first+count-1 (1-based), on all host threads."""
    stamps = []
    t0 = time.perf_counter()
    run(lambda prob, sweep, **k: stamps.append(time.perf_counter()))
    marks = [t0] + stamps
    return marks[first - 1 + count] - marks[first - 1]


def run_c1(args):
    """The reference's own CPU-runnable case: Heisenberg N=20, random MPS bond dimension
    10 from seed 0, 2-site DMRG, maxdim 64, cutoff 1e-10, Lanczos krylovdim 3 / maxiter 1.
    One step = one sweep (W warm-up sweeps, K timed)."""
    import networksolvers_gb300 as ns
    import networksolvers_gb300.models as m
    from networksolvers_gb300 import _native
    ctx = _native.Context(0, precision=args.precision)
    _native.set_default_context(ctx)
    H, psi0 = m.config_heisenberg_chain(20, 10, 0)
    kw = dict(nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
              inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=64)))
    total = args.warmup + args.steps
    marks = []
    ctx.synchronize()

    def cb(prob, sweep, **k):
        ctx.record(sweep % 2)
        ctx.synchronize()
        marks.append(time.perf_counter())

    t0 = time.perf_counter()
    E, _ = ns.dmrg(H, psi0, nsweeps=total, sweep_callback=cb, **kw)
    marks = [t0] + marks
    t = marks[total] - marks[args.warmup]
    cpu = None
    if not args.no_cpu:
        from oracle import sweep as osw
        tc = _oracle_sweep_seconds(lambda cbk: osw.dmrg(H, psi0, nsweeps=total, sweep_callback=cbk, **kw),
                                   args.warmup + 1, args.steps)
        cpu = {"value": args.steps / tc, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"the same run, sweeps {args.warmup + 1}-{total}"}
    _line(metric="dmrg_sweeps_per_s", value=args.steps / t, unit="sweeps/s", steps=args.steps, warmup=args.warmup,
          ms_per_step=t * 1e3 / args.steps, dtype="f64" if args.precision == "fp64" else f"{args.precision}+f64",
          config={"workload": "heisenberg_chain_N20_2site_dmrg_maxdim64", "timing": "host clock around synchronised sweeps"},
          energy=E, cpu_baseline=cpu)


def run_tdvp(args):
    """2-site TDVP on the depth-5 binary-tree TFIM (63 sites, d=2, complex128): all-up
    start, dt = 0.05, maxdim 256, cutoff 1e-9, Krylov exponential tol 1e-12.  One step =
    one time step (a 4th-order TDVP sweep).  The split form is timed over steps
    W+1..W+K and compared with the plain form over the same steps (fidelity of the two
    final states)."""
    import networksolvers_gb300.models as m
    from networksolvers_gb300 import _native
    from networksolvers_gb300.network import inner
    from networksolvers_gb300.sweep import ApplyExpProblem, exponentiate_solver, sweep_solve, updater_applyexp
    from networksolvers_gb300.network import tdvp_regions
    ctx = _native.Context(0, precision="fp64")
    _native.set_default_context(ctx)
    g = m.binary_tree_graph(5)
    H = m.tfim_tree(g, h=1.0).astype(np.complex128)
    psi0 = m.all_up_state(g)
    trunc = dict(cutoff=1e-9, maxdim=256)
    total = args.warmup + args.steps
    from networksolvers_gb300.network import ProjTTN, from_network
    out = {}
    sites = {}  # both runs share the site indices, so their final states can be overlapped
    for prec in ("fp64", args.precision):
        ctx.set_precision(prec)
        psi, _ = from_network(psi0, site_index=sites, ctx=ctx, dtype=np.complex128)
        (gh, Ht), _ = from_network(H, site_index=sites, ctx=ctx, dtype=np.complex128)
        P = ProjTTN(psi.g, Ht)
        prob = ApplyExpProblem(psi, P)
        ms = []
        for step in range(total):
            plan = tdvp_regions(psi.g, -1j * 0.05, updater_kwargs=dict(solver=exponentiate_solver, tol=1e-12),
                                tdvp_order=4, nsites=2, inserter_kwargs=dict(trunc=trunc))
            ctx.synchronize()
            ctx.record(0)
            prob = sweep_solve(prob, [plan], updater_applyexp)
            ctx.record(1)
            ms.append(ctx.elapsed_ms(0, 1))
        out[prec] = (prob.state, ms[args.warmup:], prob.state.maxlinkdim())
    cpu = None
    if not args.no_cpu:
        from oracle import sweep as osw
        exps = [-1j * 0.05 * k for k in range(total + 1)]
        tc = _oracle_sweep_seconds(
            lambda cbk: osw.applyexp(H, psi0, exps, nsites=2, sweep_callback=cbk,
                                     updater_kwargs=dict(solver=osw.exponentiate_solver, tol=1e-12),
                                     inserter_kwargs=dict(trunc=trunc)), args.warmup + 1, args.steps)
        cpu = {"value": args.steps / tc, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"the same run, steps {args.warmup + 1}-{total}"}
    a, b = out["fp64"][0], out[args.precision][0]
    ab, aa, bb = inner(a, b), inner(a, a), inner(b, b)
    fid = abs(ab) ** 2 / (abs(aa) * abs(bb))
    t = float(np.sum(out[args.precision][1])) / 1e3
    tp = float(np.sum(out["fp64"][1])) / 1e3
    _line(metric="tdvp_steps_per_s", value=args.steps / t, unit="steps/s", steps=args.steps, warmup=args.warmup,
          ms_per_step=t * 1e3 / args.steps, dtype=f"c128 ({args.precision})",
          config={"workload": "tfim_binary_tree_depth5_2site_tdvp", "sites": 63, "dt": 0.05, "maxdim": 256,
                  "cutoff": 1e-9, "timed_steps": list(range(args.warmup + 1, total + 1))},
          plain_fp64={"value": args.steps / tp, "unit": "steps/s"}, split_vs_plain=tp / t,
          fidelity_split_vs_plain=fid, maxlinkdim=out[args.precision][2], cpu_baseline=cpu)


def run_c3_accuracy(args):
    """The large DMRG configuration run to its full --sweeps (10) sweeps in several forms from
    the same initial state (--forms, default "fp64,ozaki"; "fp64p" is the plain form from
    the initial state perturbed by 1e-13 relative noise, a measure of how far rounding-level
    differences carry through the truncations).  Per form: the energy after every sweep and
    every region, the truncated bond dimension of every region, per-sweep times (CUDA
    events) and the time to solution; against the plain form: |dE/E| per sweep and the
    first region whose bond dimension differs."""
    import networksolvers_gb300 as ns
    from networksolvers_gb300 import _native
    from networksolvers_gb300.models import Network
    ctx = _native.Context(0, precision="fp64")
    _native.set_default_context(ctx)
    H, psi0 = workload()
    kw = kwargs_for(0)
    forms = [f for f in args.forms.split(",") if f]
    if "fp64" not in forms:
        forms = ["fp64"] + forms
    res = {}
    for form in forms:
        prec = "fp64" if form == "fp64p" else form
        start = psi0
        if form == "fp64p":
            rng = np.random.Generator(np.random.PCG64(12345))
            start = Network(psi0.graph, {v: t * (1.0 + 1e-13 * rng.standard_normal(t.shape))
                                         for v, t in psi0.tensors.items()}, psi0.legs, np.float64, dict(psi0.meta))
        ctx.set_precision(prec)
        ens, ms, regs = [], [], []
        ctx.synchronize()
        ctx.record(0)

        def cb(prob, sweep, **k):
            ctx.record(1)
            ms.append(ctx.elapsed_ms(0, 1))
            ctx.record(0)
            ens.append(prob.eigenvalue)

        def rcb(prob, sweep, region, which, **k):
            regs.append((sweep, which, prob.eigenvalue, prob.last_insert.get("newdim", -1),
                         prob.last_insert.get("truncerr", 0.0)))

        E, psi = ns.dmrg(H, start, nsweeps=args.sweeps, sweep_callback=cb, region_callback=rcb, **kw)
        res[form] = dict(energies=ens, sweep_ms=ms, regions=np.array(regs), maxlinkdim=psi.maxlinkdim())
    ref = res["fp64"]
    out = {}
    for form, r in res.items():
        d = dict(energy=r["energies"][-1], time_to_solution_s=float(np.sum(r["sweep_ms"])) / 1e3,
                 sweep_ms=r["sweep_ms"], energies=r["energies"], maxlinkdim=r["maxlinkdim"])
        if form != "fp64":
            d["rel_dE_per_sweep"] = [abs(a - b) / abs(b) for a, b in zip(r["energies"], ref["energies"])]
            diff = np.nonzero(r["regions"][:, 3] != ref["regions"][:, 3])[0]
            d["first_bond_difference"] = (None if len(diff) == 0 else
                                          {"index": int(diff[0]), "sweep": int(r["regions"][diff[0], 0]),
                                           "region": int(r["regions"][diff[0], 1]),
                                           "newdim": int(r["regions"][diff[0], 3]),
                                           "newdim_fp64": int(ref["regions"][diff[0], 3]),
                                           "truncerr": float(r["regions"][diff[0], 4]),
                                           "truncerr_fp64": float(ref["regions"][diff[0], 4])})
            d["regions_with_bond_difference"] = int(len(diff))
            rel = np.abs(r["regions"][:, 2] - ref["regions"][:, 2]) / np.abs(ref["regions"][:, 2])
            d["max_region_rel_dE_before_first_bond_difference"] = float(np.max(rel[:diff[0]])) if len(diff) else \
                float(np.max(rel))
            d["speedup_vs_fp64"] = float(np.sum(ref["sweep_ms"])) / float(np.sum(r["sweep_ms"]))
        out[form] = d
    main_form = [f for f in forms if f not in ("fp64", "fp64p")]
    mf = main_form[0] if main_form else "fp64"
    _line(metric="dmrg_energy_agreement", value=out[mf].get("rel_dE_per_sweep", [0.0])[-1], unit="|dE/E|",
          higher_is_better=False, steps=args.sweeps, warmup=0,
          ms_per_step=float(np.mean(res[mf]["sweep_ms"])), dtype=f"{mf}+f64 vs f64",
          config={"workload": "heisenberg_chain_N100_2site_dmrg_maxdim1024", "sweeps": args.sweeps,
                  "maxdim_schedule": SCHEDULE, "cutoff": CUTOFF, "forms": forms},
          forms=out)


def _pool_jobs_c4(count):
    import networksolvers_gb300.models as m
    from networksolvers_gb300 import batch
    jobs = []
    for k in range(count):
        c = m.config_j1j2_batch(k)
        jobs.append(batch.dmrg_job(c["H"], c["psi0"], tag=k, nsweeps=6, maxdim=c["maxdim"], cutoff=1e-10))
    return jobs


def run_batch(args):
    """256 independent J1-J2 chains (seed k: N~U[16,64], J2~U[0,0.5], maxdim~U{32,64,128},
    random MPS bond dimension 8, 6 sweeps, cutoff 1e-10) advanced concurrently by a pool
    of workers (one context and stream each), against sequential plain FP64 solves of
    the first --sample chains (the same chains' energies give the accuracy)."""
    from networksolvers_gb300 import batch
    jobs = _pool_jobs_c4(args.chains)
    t0 = time.perf_counter()
    seq = batch.SolvePool(workers=1, precision="fp64").run(jobs[:args.sample])
    t_seq = time.perf_counter() - t0
    tuning = {k: v for k, v in (("tridiag", args.pool_tridiag), ("dc_leaf", args.pool_leaf)) if v} or None
    pool = batch.SolvePool(workers=args.workers, precision=args.precision, tuning=tuning)
    t0 = time.perf_counter()
    res = pool.run(jobs)
    t_pool = time.perf_counter() - t0
    err = [r.error for r in res + seq if r.error]
    dE = max(abs(r.value - q.value) / abs(q.value) for r, q in zip(res, seq))
    v = len(res) / t_pool
    cpu = None
    if not args.no_cpu:
        from oracle import sweep as osw
        t0 = time.perf_counter()
        ncpu = 2
        for j in jobs[:ncpu]:
            kw = dict(j.kwargs)
            osw.dmrg(j.H, j.psi0, kw.pop("nsweeps"), **kw)
        tc = time.perf_counter() - t0
        cpu = {"value": ncpu / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "chains 0-1, sequential"}
    _line(metric="batched_dmrg_solves_per_s", value=v, unit="solves/s", steps=1, warmup=0,
          ms_per_step=t_pool * 1e3, dtype=f"f64 ({args.precision})",
          config={"workload": "j1j2_chain_batch", "chains": len(jobs), "workers": args.workers,
                  "nsweeps": 6, "cutoff": 1e-10, "tuning": tuning or "table"},
          gpu_launches=pool.launches, launches_per_s=pool.launches / t_pool,
          sequential_fp64={"value": args.sample / t_seq, "unit": "solves/s", "sample": f"chains 0..{args.sample - 1}"},
          speedup_vs_sequential=v / (args.sample / t_seq), max_rel_dE_vs_sequential=dE, errors=err[:3],
          cpu_baseline=cpu)


def _serve_jobs(rate, duration, seed):
    import networksolvers_gb300.models as m
    from networksolvers_gb300 import batch
    arr = batch.poisson_arrivals(rate, duration, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    jobs = []
    for i, t in enumerate(arr):
        if rng.uniform() < 0.7:
            n = int(rng.integers(20, 129))
            delta = float(rng.uniform(0.0, 2.0))
            md = int(rng.choice([64, 128, 256]))
            H = m.xxz_chain(n, delta)
            psi0 = m.random_state(m.chain_graph(n), 8, seed=seed * 100003 + i)
            jobs.append(batch.dmrg_job(H, psi0, tag=("dmrg", i), arrival=t, nsweeps=5, maxdim=md, cutoff=1e-10))
        else:
            depth = int(rng.integers(3, 6))
            h = float(rng.uniform(0.5, 1.5))
            g = m.binary_tree_graph(depth)
            H = m.tfim_tree(g, h=h).astype(np.complex128)
            jobs.append(batch.tdvp_job(H, m.all_up_state(g), [0.05 * (k + 1) for k in range(20)], tag=("tdvp", i),
                                       arrival=t, maxdim=64))
    return jobs


def run_serve(args):
    """Serving stream: Poisson arrivals at --rate req/s for --duration s (seeded), 70 %
    ground-state DMRG on XXZ chains (N~U[20,128], Delta~U[0,2], maxdim~U{64,128,256},
    5 sweeps, cutoff 1e-10), 30 % TDVP quenches of binary-tree TFIM (depth 3-5,
    h~U[0.5,1.5], 20 steps of dt=0.05, maxdim 64).  Admission by HBM footprint;
    p50 / p99 latency and solves/s, against sequential plain FP64 solves of the first
    --sample requests."""
    from networksolvers_gb300 import batch
    jobs = _serve_jobs(args.rate, args.duration, args.seed)
    t0 = time.perf_counter()
    seq = batch.SolvePool(workers=1, precision="fp64").run(
        [batch.Job(j.kind, j.H, j.psi0, j.kwargs, j.tag, 0.0) for j in jobs[:args.sample]])
    t_seq = time.perf_counter() - t0
    res = batch.SolvePool(workers=args.workers, precision=args.precision).run(jobs)
    summ = batch.latency_summary(res)
    same = []
    for r, q in zip(res, seq):
        if r.kind == "dmrg" and r.error is None and q.error is None:
            same.append(abs(r.value - q.value) / abs(q.value))
    _line(metric="served_solves_per_s", value=summ["solves_per_s"], unit="solves/s", steps=1, warmup=0,
          ms_per_step=summ["span_s"] * 1e3, dtype=f"f64/c128 ({args.precision})",
          config={"workload": "serve_xxz_dmrg_tfim_tdvp_mix", "rate_per_s": args.rate, "duration_s": args.duration,
                  "requests": len(jobs), "workers": args.workers},
          latency={"p50_s": summ["p50_s"], "p99_s": summ["p99_s"]}, failed=summ["failed"],
          sequential_fp64={"value": args.sample / t_seq, "unit": "solves/s",
                           "sample": f"requests 0..{args.sample - 1}"},
          max_rel_dE_vs_sequential=max(same) if same else None)


def run_serve_sweep(args):
    """The serving mix (see run_serve) offered at increasing Poisson rates (--rates), a
    fixed number of requests (--requests) per rate, so each rate's arrival window is
    requests / rate seconds.  Per rate: achieved solves/s, p50 / p99 latency, mean and
    largest queue wait (admission delay), against the configured 200 req/s.  The
    sustainable rate is the plateau of the achieved throughput over the offered rates
    (above it, requests queue and latency grows with the length of the stream).
    Beside it: sequential plain FP64 solves of the first --sample requests of the
    lowest rate."""
    from networksolvers_gb300 import batch
    rates = [float(r) for r in args.rates.split(",") if r]
    rows = []
    seq_rate = None
    for k, rate in enumerate(rates):
        jobs = _serve_jobs(rate, args.requests / rate, args.seed + k)
        if k == 0 and args.sample > 0:
            t0 = time.perf_counter()
            batch.SolvePool(workers=1, precision="fp64").run(
                [batch.Job(j.kind, j.H, j.psi0, j.kwargs, j.tag, 0.0) for j in jobs[:args.sample]])
            seq_rate = args.sample / (time.perf_counter() - t0)
        res = batch.SolvePool(workers=args.workers, precision=args.precision).run(jobs)
        summ = batch.latency_summary(res)
        ok = [r for r in res if r.error is None]
        waits = np.array([r.start - r.arrival for r in ok]) if ok else np.zeros(1)
        service = np.array([r.finish - r.start for r in ok]) if ok else np.zeros(1)
        rows.append({"offered_per_s": rate, "requests": len(jobs), "achieved_per_s": summ["solves_per_s"],
                     "p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "mean_wait_s": float(np.mean(waits)),
                     "max_wait_s": float(np.max(waits)), "median_service_s": float(np.median(service)),
                     "failed": summ["failed"]})
        print(json.dumps({"progress": rows[-1]}), file=sys.stderr, flush=True)
    # the pool saturates where the achieved throughput stops growing with the offered
    # rate: that plateau is the sustainable rate (offered rates above it build a backlog)
    peak = max((r["achieved_per_s"] or 0.0) for r in rows)
    sustainable = peak
    _line(metric="served_solves_per_s", value=peak, unit="solves/s", steps=len(rows), warmup=0,
          ms_per_step=None, dtype=f"f64/c128 ({args.precision})",
          config={"workload": "serve_xxz_dmrg_tfim_tdvp_mix", "configured_rate_per_s": 200.0, "rates": rates,
                  "requests_per_rate": args.requests, "workers": args.workers},
          rates=rows, sustainable_rate_per_s=sustainable,
          sequential_fp64={"value": seq_rate, "unit": "solves/s", "sample": f"first {args.sample} requests"})


def run_qn(args):
    """U(1) block-sparse DMRG (the `conserve_qns=true` path): Heisenberg chain N=40 from the
    Neel state, 2-site, maxdim [32, 64, 128, 256] then 256, cutoff 1e-10, Lanczos krylovdim
    3 / maxiter 1; one step = one sweep (W warm-up sweeps, K timed, host clock around
    synchronised sweeps).  Beside it: the dense GPU chain driver on the same run, and the
    dense CPU oracle on its sweeps 1..W+1 (sample)."""
    import networksolvers_gb300.models as m
    from networksolvers_gb300 import _native, qn
    from networksolvers_gb300.chain import dmrg_chain
    ctx = _native.Context(0, precision=args.precision)
    _native.set_default_context(ctx)
    n = 40
    H = m.heisenberg_chain(n)
    g = m.chain_graph(n)
    states = [0 if v % 2 else 1 for v in range(1, n + 1)]
    psi0 = m.product_state(g, {v: ("Up" if v % 2 else "Dn") for v in g.vertices})
    total = args.warmup + args.steps
    kw = dict(maxdim=[32, 64, 128, 256], cutoff=1e-10, krylovdim=3, maxiter=1)
    nreg = 2 * (n - 1)

    def timed(run):
        marks = []

        def cb(sweep, k, energy, info):
            if k == nreg - 1:
                ctx.synchronize()
                marks.append(time.perf_counter())

        ctx.synchronize()
        t0 = time.perf_counter()
        out = run(cb)
        marks = [t0] + marks
        return out, marks[total] - marks[args.warmup]

    (Eq, A, rq), tq = timed(lambda cb: qn.qn_dmrg_chain(H, states, total, ctx=ctx, region_callback=cb, **kw))
    (Ed, _, rd), td = timed(lambda cb: dmrg_chain(H, psi0, total, ctx=ctx, region_callback=cb, **kw))
    nnz = sum(t.nnz() for t in A)
    dense_size = sum(int(np.prod([q.dim for q in t.inds])) for t in A)
    cpu = None
    if not args.no_cpu:
        from oracle import sweep as osw
        okw = dict(nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
                   inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=kw["maxdim"])))
        sample = args.warmup + 1
        tc = _oracle_sweep_seconds(lambda cbk: osw.dmrg(H, psi0, nsweeps=sample, sweep_callback=cbk, **okw),
                                   sample, 1)
        cpu = {"value": 1.0 / tc, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"dense oracle, sweep {sample} of the same schedule"}
    _line(metric="qn_dmrg_sweeps_per_s", value=args.steps / tq, unit="sweeps/s", steps=args.steps,
          warmup=args.warmup, ms_per_step=tq * 1e3 / args.steps,
          dtype="f64" if args.precision == "fp64" else f"{args.precision}+f64",
          config={"workload": "heisenberg_chain_N40_2site_qn_dmrg_maxdim256", "start": "Neel", "cutoff": 1e-10,
                  "timing": "host clock around synchronised sweeps"},
          energy=Eq, dense_gpu={"value": args.steps / td, "unit": "sweeps/s", "energy": Ed,
                                "rel_dE": abs(Eq - Ed) / abs(Ed),
                                "bond_dims_equal": [r[3] for r in rq] == [r[3] for r in rd]},
          block_sparse_fraction=nnz / dense_size, maxlinkdim=max(r[3] for r in rq), cpu_baseline=cpu)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nsg", choices=["nsg", "reference"])
    ap.add_argument("--precision", default="ozaki", choices=["ozaki", "tf32x3", "fp64"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="dmrg", choices=["dmrg", "c1", "tdvp", "batch", "serve", "serve_sweep", "accuracy", "qn"],
                    help="dmrg: the N=100 benchmark (default); c1: the N=20 chain; tdvp: binary-tree TFIM "
                         "TDVP; batch: 256 J1-J2 chains on a solve pool; serve: Poisson request stream; "
                         "qn: U(1) block-sparse DMRG")
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--pool-tridiag", type=int, default=0,
                    help="batch: the workers' reduction path (-1 grid kernel, 2-16 cluster size, 0 the table)")
    ap.add_argument("--pool-leaf", type=int, default=16,
                    help="batch: the workers' divide-and-conquer leaf order (4-32; 0 the single-solve default "
                         "of 8; 16, fewer launches per eigensolve, measured the better throughput choice)")
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--sample", type=int, default=16)
    ap.add_argument("--rate", type=float, default=1.0)
    ap.add_argument("--duration", type=float, default=30.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rates", default="0.25,0.5,1,2,4", help="serve_sweep: offered request rates")
    ap.add_argument("--requests", type=int, default=24, help="serve_sweep: requests per rate")
    ap.add_argument("--sweeps", type=int, default=10)
    ap.add_argument("--forms", default="fp64,ozaki", help="accuracy workload: forms to run (fp64, ozaki, "
                                                          "ozaki8, tf32x3, fp64p)")
    args = ap.parse_args()
    if args.warmup < 3 and args.workload in ("dmrg", "c1", "tdvp", "qn"):
        raise SystemExit("warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c1":
        run_c1(args)
    elif args.workload == "accuracy":
        run_c3_accuracy(args)
    elif args.workload == "tdvp":
        run_tdvp(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "serve_sweep":
        run_serve_sweep(args)
    elif args.workload == "qn":
        run_qn(args)
    else:
        run_nsg(args)


if __name__ == "__main__":
    main()
