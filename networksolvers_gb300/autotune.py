"""Autotuner of the library's launch choices; writes the compiled-in tuning table.

    python -m networksolvers_gb300.autotune [--out DIR] [--reps 5]

Measures on the current GPU, with per-context overrides (nsg_ctx_set_tuning) and CUDA
events around the kernels of the class (nsg_ctx_profile):

* the Householder tridiagonalisation of the truncated factorization, for matrix orders
  32..576: the grid-wide cooperative kernel against one thread-block cluster of 2, 4, 8
  and 16 CTAs (where the matrix fits the cluster's shared memory);
* the FP64 CUDA-core GEMM of small outputs (the eigensolver's products at small bond
  dimension), for output sizes 32..256 and depths 64..4096: split K into 1..64 slices.

For each case the fastest choice (median of --reps) goes into DIR/tuning.json and
DIR/tuning_table.h (the header the library compiles in: copy it to
networksolvers_gb300/csrc/ and rebuild).  Orders whose best path is the grid kernel end
the cluster table; split-K buckets whose best count equals the built-in rule's are kept
too (the table then pins what was measured).
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

TRI_ORDERS = [32, 48, 64, 96, 128, 192, 256, 320, 384, 448, 512, 576]
TRI_PATHS = [-1, 2, 4, 8, 16]
GEMM_SIZES = [32, 64, 128, 256]
GEMM_DEPTHS = [64, 128, 256, 512, 1024, 2048, 4096]
SPLITS = [1, 2, 4, 8, 16, 32, 64]


def cluster_fits(n, C, elem=8, cap=200 * 1024):
    return ((n + C - 1) // C * n + 4 * n) * elem <= cap


def _median_class_ms(ctx, cls, run, reps):
    out = []
    run()  # warm-up (and any one-time set-up)
    for _ in range(reps):
        ctx.synchronize()
        ctx.profile(True)
        run()
        prof = ctx.profile_read()
        ctx.profile(False)
        out.append(prof[cls]["ms"])
    return float(np.median(out))


def tune_tridiag(ctx, reps):
    from .itensors import DTensor, Index, factorize
    rng = np.random.default_rng(3)
    rows = []
    for n in TRI_ORDERS:
        M = rng.standard_normal((n, n))
        l, r = Index(n), Index(n)
        T = DTensor.from_numpy(M, [l, r])
        times = {}
        for path in TRI_PATHS:
            if path > 0 and not cluster_fits(n, path):
                continue
            ctx.set_tuning("tridiag", path)
            times[path] = _median_class_ms(ctx, "tridiag", lambda: factorize(T, [l], cutoff=1e-12, maxdim=n // 2),
                                           reps)
        ctx.set_tuning("tridiag", 0)
        best = min(times, key=times.get)
        rows.append({"order": n, "ms": {str(k): v for k, v in times.items()}, "best": best})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    return rows


def tune_splitk(ctx, reps):
    from .itensors import DTensor, Index, contract
    rng = np.random.default_rng(4)
    rows = []
    for m in GEMM_SIZES:
        for k in GEMM_DEPTHS:
            i, j, l = Index(m), Index(m), Index(k)
            A = DTensor.from_numpy(rng.standard_normal((m, k)), [i, l])
            B = DTensor.from_numpy(rng.standard_normal((k, m)), [l, j])
            times = {}
            for sp in SPLITS:
                if sp > max(1, k // 16):
                    continue
                ctx.set_tuning("splitk", sp)
                times[sp] = _median_class_ms(ctx, "simt_gemm", lambda: contract([A, B], out=[i, j]), reps)
            ctx.set_tuning("splitk", 0)
            auto = _median_class_ms(ctx, "simt_gemm", lambda: contract([A, B], out=[i, j]), reps)
            best = min(times, key=times.get)
            tiles = ((m + 63) // 64) ** 2
            rows.append({"m": m, "n": m, "k": k, "tiles": tiles, "ms": {str(s): v for s, v in times.items()},
                         "rule_ms": auto, "best": best})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    return rows


def tri_entries(rows):
    """(max_order, path) entries: consecutive orders with the same best cluster size
    merged; the table ends before the first order whose best path is the grid kernel."""
    out = []
    for r in rows:
        if r["best"] == -1:
            break
        if out and out[-1][1] == r["best"]:
            out[-1] = (r["order"], r["best"])
        else:
            out.append((r["order"], r["best"]))
    return out


def split_entries(rows):
    """(max_tiles, max_k, splits) entries in increasing (tiles, k): first match wins.
    Output sizes that fall in the same tile count (32 and 64 both make one 64 x 64 tile)
    share a bucket, whose split count is the one with the least summed time over them."""
    groups = {}
    for r in rows:
        groups.setdefault((r["tiles"], r["k"]), []).append(r["ms"])
    out = []
    for key in sorted(groups):
        ms = groups[key]
        common = set(ms[0]).intersection(*ms[1:])
        best = min(common, key=lambda s: sum(t[s] for t in ms))
        out.append((key[0], key[1], int(best)))
    return out


def header(tri, split, device_name):
    lines = [
        "// Tuning table of the library's launch choices, written by the autotuner",
        "// (python -m networksolvers_gb300.autotune, which measures every candidate on the GPU and",
        "// writes this file and networksolvers_gb300/tuning.json).  Compiled in; a context can",
        "// override an entry for measurement (nsg_ctx_set_tuning).",
        f"// Measured on: {device_name}.",
        "#pragma once",
        "",
        "namespace nsg {",
        "namespace tuning {",
        "",
        "// Householder tridiagonalisation by matrix order: orders up to max_order use `path`",
        "// (2..16: one thread-block cluster of that many CTAs; 0: the grid-wide cooperative",
        "// kernel).  Orders above the last entry use the grid kernel.",
        "struct TriEntry {",
        "  int max_order;",
        "  int path;",
        "};",
        "constexpr TriEntry kTri[] = {",
        "    " + " ".join(f"{{{a}, {b}}}," for a, b in (tri or [(0, 0)])),
        "};",
        "",
        "// FP64 CUDA-core GEMM: number of K slices (split K) for products whose output has",
        "// `tiles` 64 x 64 tiles (times the batch) and depth K, by buckets (tiles <= max_tiles",
        "// and K <= max_k, first match); 0 keeps the built-in rule (about two slices per SM).",
        "struct SplitEntry {",
        "  int max_tiles;",
        "  int max_k;",
        "  int splits;",
        "};",
        "constexpr SplitEntry kSplit[] = {",
    ]
    for a, b, c in (split or [(0, 0, 0)]):
        lines.append(f"    {{{a}, {b}, {c}}},")
    lines += ["};", "", "}  // namespace tuning", "}  // namespace nsg", ""]
    return "\n".join(lines)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m networksolvers_gb300.autotune")
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--from-json", default=None,
                    help="rewrite the tables from a tuning.json of an earlier run, measuring nothing")
    args = ap.parse_args(argv)
    if args.from_json:
        d = json.loads(Path(args.from_json).read_text())
        return _write(Path(args.out), d["device"], d["tridiag"], d["splitk"])
    from . import _native
    from .build import build
    build()
    ctx = _native.Context(0, precision="fp64")
    _native.set_default_context(ctx)
    try:
        import subprocess
        dev = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                             text=True).stdout.strip().splitlines()[0]
    except Exception:
        dev = "unknown GPU"
    tri_rows = tune_tridiag(ctx, args.reps)
    split_rows = tune_splitk(ctx, args.reps)
    return _write(Path(args.out), dev, tri_rows, split_rows)


def _write(out, dev, tri_rows, split_rows):
    tri, split = tri_entries(tri_rows), split_entries(split_rows)
    out.mkdir(parents=True, exist_ok=True)
    (out / "tuning.json").write_text(json.dumps({"device": dev, "tridiag": tri_rows, "splitk": split_rows,
                                                 "table": {"tridiag": tri, "splitk": split}}, indent=1) + "\n")
    (out / "tuning_table.h").write_text(header(tri, split, dev))
    print(json.dumps({"tridiag": tri, "splitk": split}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
