// Tuning table of the library's launch choices, written by the autotuner
// (python -m networksolvers_gb300.autotune, which measures every candidate on the GPU and
// writes this file and networksolvers_gb300/tuning.json).  Compiled in; a context can
// override an entry for measurement (nsg_ctx_set_tuning).
// Measured on: NVIDIA GB300.
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
    {48, 8}, {384, 16},
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
    {1, 64, 4},
    {1, 128, 8},
    {1, 256, 16},
    {1, 512, 32},
    {1, 1024, 64},
    {1, 2048, 64},
    {1, 4096, 64},
    {4, 64, 4},
    {4, 128, 8},
    {4, 256, 16},
    {4, 512, 32},
    {4, 1024, 32},
    {4, 2048, 32},
    {4, 4096, 64},
    {16, 64, 4},
    {16, 128, 8},
    {16, 256, 16},
    {16, 512, 16},
    {16, 1024, 64},
    {16, 2048, 64},
    {16, 4096, 64},
};

}  // namespace tuning
}  // namespace nsg
