"""Many independent solves on one GPU: a pool of workers that advance DMRG and TDVP
solves concurrently, admission by HBM footprint, and a continuous-batching server loop.

Each worker thread owns a library context (its own CUDA stream, memory accounting and
device error flag) and runs the same drivers as a single solve (`eigsolve` /
`applyexp`, eigsolve.jl:45-76 / applyexp.jl:62-103), so a solve's result does not depend
on what else is in flight: every kernel of a solve is ordered on that solve's stream,
and the kernels are deterministic.  The host parts of the drivers run between library
calls (which release the interpreter lock); the GPU work of the workers overlaps on the
device.

`SolvePool.run(jobs)` admits jobs in arrival order as soon as a worker is free and the
estimated device footprint of the running jobs plus the new one fits the HBM budget
(head-of-line: a job that does not fit waits for memory to free up), and records for
every job its arrival, start and finish times.  With every arrival at 0 this is the
batched throughput mode; with Poisson arrivals (`poisson_arrivals`) it is the serving
mode, and `latency_summary` gives p50 / p99 latency and solves/s.
"""
from __future__ import annotations

import math
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _native

__all__ = ["Job", "JobResult", "SolvePool", "footprint_bytes", "poisson_arrivals", "latency_summary",
           "dmrg_job", "tdvp_job"]


@dataclass
class Job:
    kind: str                  # "dmrg" or "tdvp"
    H: object                  # models.Network operator
    psi0: object               # models.Network initial state
    kwargs: dict               # driver keyword arguments (nsweeps / time_points, trunc, ...)
    tag: object = None
    arrival: float = 0.0       # seconds after the start of the run
    footprint: int = 0         # estimated device bytes (footprint_bytes when 0)


@dataclass
class JobResult:
    tag: object
    kind: str
    value: object              # DMRG: final energy; TDVP: dict of site tensors (numpy)
    arrival: float
    start: float
    finish: float
    worker: int
    footprint: int
    error: str = None

    @property
    def latency(self):
        return self.finish - self.arrival


def _max_maxdim(kwargs):
    md = 0
    for key in ("inserter_kwargs", "extracter_kwargs"):
        tr = (kwargs.get(key) or {}).get("trunc") or {}
        m = tr.get("maxdim")
        if m is None:
            continue
        md = max(md, max(m) if isinstance(m, (list, tuple)) else int(m))
    return md or 64


def footprint_bytes(job: Job) -> int:
    """Device bytes a solve holds at its peak: the state and the environments at the
    largest bond dimension (maxdim), plus the largest region's working set (two-site
    tensor, Krylov basis, H_eff intermediates, Gram matrix and eigensolver workspace)."""
    H, psi = job.H, job.psi0
    nsites = len(psi.graph.vertices)
    chi = _max_maxdim(job.kwargs)
    d = 2
    w = max(max(t.shape) for t in H.tensors.values())
    degree = max(len(psi.graph.neighbors(v)) for v in psi.graph.vertices)
    elem = 16 if (job.kind == "tdvp" or any(np.iscomplexobj(t) for t in H.tensors.values())) else 8
    site = d * chi ** max(degree, 1)
    state = nsites * site
    envs = 2 * nsites * w * chi * chi
    region = d * site
    kry = (32 if job.kind == "tdvp" else 5) * region
    heff = 2 * w * d * d * region
    gram = 4 * (d * chi) ** 2
    return int(elem * (state + envs + kry + heff + gram) * 1.25) + (64 << 20)


def dmrg_job(H, psi0, tag=None, arrival=0.0, nsweeps=6, maxdim=64, cutoff=1e-10, krylovdim=3, maxiter=1):
    trunc = dict(cutoff=cutoff, maxdim=maxdim)
    kw = dict(nsweeps=nsweeps, nsites=2, updater_kwargs=dict(krylovdim=krylovdim, maxiter=maxiter),
              inserter_kwargs=dict(trunc=trunc))
    return Job("dmrg", H, psi0, kw, tag, arrival)


def tdvp_job(H, psi0, time_points, tag=None, arrival=0.0, maxdim=64, cutoff=1e-9, tol=1e-12):
    from .sweep import exponentiate_solver
    trunc = dict(cutoff=cutoff, maxdim=maxdim)
    kw = dict(time_points=list(time_points), nsites=2,
              updater_kwargs=dict(solver=exponentiate_solver, tol=tol), inserter_kwargs=dict(trunc=trunc))
    return Job("tdvp", H, psi0, kw, tag, arrival)


def _is_chain(graph):
    vs = sorted(graph.vertices)
    n = len(vs)
    return vs == list(range(1, n + 1)) and all(
        sorted(graph.neighbors(v)) == [u for u in (v - 1, v + 1) if 1 <= u <= n] for v in vs)


def _run_job(job: Job, ctx):
    from .sweep import eigsolve, tdvp
    kw = dict(job.kwargs)
    if job.kind == "dmrg":
        nsweeps = kw.pop("nsweeps")
        ex = kw.get("extracter_kwargs") or {}
        if kw.get("nsites", 1) == 2 and not ex.get("subspace_algorithm") and _is_chain(job.psi0.graph):
            # plain two-site chain DMRG: the fused per-region driver (same results)
            from .chain import dmrg_chain
            up = kw.get("updater_kwargs") or {}
            tr = (kw.get("inserter_kwargs") or {}).get("trunc") or {}
            E, _, _ = dmrg_chain(job.H, job.psi0, nsweeps, maxdim=tr.get("maxdim"), cutoff=tr.get("cutoff", 0.0),
                                 mindim=tr.get("mindim", 1), krylovdim=up.get("krylovdim", 3),
                                 maxiter=up.get("maxiter", 1), tol=up.get("tol", 1e-14), ctx=ctx)
            return float(E)
        E, _ = eigsolve(job.H, job.psi0, nsweeps, ctx=ctx, **kw)
        return float(E)
    if job.kind == "tdvp":
        tp = kw.pop("time_points")
        psi = tdvp(job.H, job.psi0, tp, ctx=ctx, **kw)
        return psi.to_numpy(job.psi0)
    raise ValueError(f"unknown job kind {job.kind!r}")


class SolvePool:
    """`workers` concurrent solves on device `device`, each worker with its own context
    in precision mode `precision`; `hbm_bytes` caps the summed footprints of the running
    jobs (default: 90 % of the device's free memory at start)."""

    def __init__(self, workers=8, device=0, precision="fp64", hbm_bytes=None, context_factory=None, runner=None,
                 tuning=None):
        self.workers, self.device, self.precision = int(workers), int(device), precision
        self.hbm_bytes = hbm_bytes
        # per-worker launch-choice overrides ({"tridiag": 8, "splitk": 4}, Context.set_tuning):
        # e.g. smaller clusters for the reductions, so that more solves reduce side by side
        self.tuning = dict(tuning or {})
        self.launches = 0  # kernels launched by the workers' contexts in the last run
        # context_factory() -> context with synchronize()/close(); runner(job, ctx) -> value.
        # Defaults: a library context per worker and the DMRG / TDVP drivers.
        self._make_ctx = context_factory or (lambda: _native.Context(self.device, precision=self.precision))
        self._runner = runner or _run_job

    def run(self, jobs, time_scale=1.0):
        """Run `jobs` (arrival times in seconds, scaled by `time_scale`); returns the
        results in job order."""
        jobs = list(jobs)
        for j in jobs:
            if not j.footprint:
                j.footprint = footprint_bytes(j)
        cap = self.hbm_bytes
        if cap is None:
            cap = int(0.9 * _native.device_free_bytes(self.device))
        order = sorted(range(len(jobs)), key=lambda i: (jobs[i].arrival, i))
        results = [None] * len(jobs)
        lock = threading.Condition()
        state = {"next": 0, "in_use": 0, "running": 0}
        t0 = time.perf_counter()

        def take():
            with lock:
                while True:
                    if state["next"] >= len(order):
                        return None
                    i = order[state["next"]]
                    j = jobs[i]
                    now = time.perf_counter() - t0
                    due = j.arrival * time_scale
                    fits = state["running"] == 0 or state["in_use"] + j.footprint <= cap
                    if due <= now and fits:
                        state["next"] += 1
                        state["in_use"] += j.footprint
                        state["running"] += 1
                        return i
                    lock.wait(timeout=max(0.0, min(0.05, due - now)) if due > now else 0.05)

        def done(i):
            with lock:
                state["in_use"] -= jobs[i].footprint
                state["running"] -= 1
                lock.notify_all()

        def worker(wid):
            ctx = self._make_ctx()
            if isinstance(ctx, _native.Context):
                _native.set_thread_context(ctx)
                for param, value in self.tuning.items():
                    ctx.set_tuning(param, value)
            try:
                while True:
                    i = take()
                    if i is None:
                        break
                    j = jobs[i]
                    start = time.perf_counter() - t0
                    err, val = None, None
                    try:
                        val = self._runner(j, ctx)
                        ctx.synchronize()
                    except Exception as e:  # reported per job, the pool keeps serving
                        err = f"{type(e).__name__}: {e}"
                    finish = time.perf_counter() - t0
                    results[i] = JobResult(j.tag, j.kind, val, j.arrival * time_scale, start, finish, wid,
                                           j.footprint, err)
                    done(i)
            finally:
                _native.set_thread_context(None)
                if isinstance(ctx, _native.Context):
                    n = ctx.counters()["launches"]
                    with lock:
                        self.launches += n
                ctx.close()

        self.launches = 0
        threads = [threading.Thread(target=worker, args=(w,), daemon=True) for w in range(self.workers)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        return results


def poisson_arrivals(rate, duration, seed=0):
    """Arrival times of a Poisson process of `rate` per second over `duration` seconds."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append(t)


def latency_summary(results):
    ok = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    span = max(r.finish for r in ok) - min(r.arrival for r in ok) if ok else math.inf
    return {"solves": len(ok), "failed": len(results) - len(ok), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "solves_per_s": len(ok) / span if span > 0 else None,
            "span_s": span}
