// Tuning table of the library's launch choices, written by the autotuner
// (python -m networksolvers_gb300.autotune, which measures every candidate on the GPU and
// writes this file and networksolvers_gb300/tuning.json).  Compiled in; a context can
// override an entry for measurement (nsg_ctx_set_tuning).
#pragma once

namespace nsg {
namespace tuning {

// Householder tridiagonalisation by matrix order: orders up to max_order use `path`
// (2..16: one thread-block cluster of that many CTAs; 0: the grid-wide cooperative
// kernel).  Orders above the last entry use the grid kernel.
struct TriEntry {
  int max_order;
  int path;
};
constexpr TriEntry kTri[] = {
    {32, 2}, {64, 4}, {128, 8}, {360, 16},
};

// FP64 CUDA-core GEMM: number of K slices (split K) for products whose output has
// `tiles` 64 x 64 tiles (times the batch) and depth K, by buckets (tiles <= max_tiles
// and K <= max_k, first match); 0 keeps the built-in rule (about two slices per SM).
struct SplitEntry {
  int max_tiles;
  int max_k;
  int splits;
};
constexpr SplitEntry kSplit[] = {
    {0, 0, 0},
};

}  // namespace tuning
}  // namespace nsg
