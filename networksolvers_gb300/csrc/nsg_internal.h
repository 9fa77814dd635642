// Internal declarations shared by the nsg translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <functional>
#include <stdexcept>

#include "../../include/nsg.h"

namespace nsg {

// ---------------------------------------------------------------------------
// errors: internal code throws nsg::Error; every extern "C" entry point catches
// and turns it into a status code plus the context's last-error message.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define NSG_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      throw ::nsg::Error(NSG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define NSG_CHECK(cond, code, msg)                                                  \
  do {                                                                              \
    if (!(cond)) throw ::nsg::Error((code), (msg));                                 \
  } while (0)

struct Ctx;

}  // namespace nsg

struct nsg_tensor {
  int dtype = NSG_F64;
  int rank = 0;
  int64_t dims[NSG_MAX_RANK] = {};
  int64_t size = 1;  // number of elements
  void* data = nullptr;
  size_t bytes = 0;
};

struct nsg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0, in_use = 0, peak = 0;
  int precision = NSG_PREC_FP64;
  std::string err;
  uint64_t launches = 0, flops = 0, contractions = 0, applies = 0;
  // Krylov dimension the last exponentiate cycle used: the next cycle runs that many
  // steps without host synchronisation before it checks convergence
  int krylov_hint = 0;
  // launch-choice overrides set by nsg_ctx_set_tuning (0: the compiled-in tuning table)
  int tune_splitk = 0;  // FP64 GEMM K slices (> 0 forces that count)
  int tune_tri = 0;     // tridiagonalisation: -1 grid kernel, 2..16 cluster size
  int tune_dc_leaf = 0; // divide and conquer leaf order (4..32; 0 the default)
  // pinned host staging for scalar readback
  double* host_scalars = nullptr;
  size_t host_scalars_cap = 0;
  // device scratch for reductions
  double* dev_scratch = nullptr;
  size_t dev_scratch_cap = 0;
  int* dev_flag = nullptr;     // raised by tensor-core kernels whose bounded waits expired
  bool flag_pending = false;   // a launch since the last check may have raised it
  int num_sms = 0;
  cudaEvent_t events[16] = {};
  bool profiling = false;
  struct ProfRec {
    int cls;
    cudaEvent_t a, b;
    double flops;
  };
  std::vector<ProfRec> prof;
  bool timing = false;                           // per-phase timers (nsg_ctx_timers)
  cudaEvent_t phase_open[NSG_PHASE_NCOUNT] = {};  // start event of each open phase
  std::vector<ProfRec> phases;                   // closed intervals (cls = phase)
};

namespace nsg {

inline size_t elem_bytes(int dtype) { return dtype == NSG_C128 ? 16 : 8; }

// memory
void* dalloc(nsg_ctx* c, size_t bytes);
void dfree(nsg_ctx* c, void* p, size_t bytes);
// Device buffer from the context's pool, returned to it when the scope ends (also when
// a later step of the same call throws).
struct ScopedBuf {
  nsg_ctx* c;
  void* p = nullptr;
  size_t bytes = 0;
  ScopedBuf(nsg_ctx* cc, size_t b) : c(cc), bytes(b) { p = dalloc(c, b); }
  ~ScopedBuf() {
    try {
      dfree(c, p, bytes);
    } catch (...) {
    }
  }
  ScopedBuf(const ScopedBuf&) = delete;
  ScopedBuf& operator=(const ScopedBuf&) = delete;
};
nsg_tensor* new_tensor(nsg_ctx* c, int dtype, int rank, const int64_t* dims, bool zero = false);
void free_tensor(nsg_ctx* c, nsg_tensor* t);
double* host_scalars(nsg_ctx* c, size_t n);
double* dev_scratch(nsg_ctx* c, size_t n);
// The context's device error flag (zeroed on creation).  Kernels that may time out
// write 1 into it instead of forcing a synchronisation per launch; every public entry
// point checks it once at its end (check_device_flag) and reports NSG_ERR_TIMEOUT.
int* device_flag(nsg_ctx* c);
void check_device_flag(nsg_ctx* c);
inline void count_launch(nsg_ctx* c, int n = 1) { c->launches += n; }

// Brackets a kernel launch with CUDA events while the context is profiling.
struct ProfScope {
  nsg_ctx* c;
  int cls;
  double flops;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(nsg_ctx* cc, int k, double f) : c(cc), cls(k), flops(f) {
    if (c->profiling) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, c->stream);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEventRecord(b, c->stream);
      c->prof.push_back({cls, a, b, flops});
    }
  }
};
// Brackets a phase of the region step with CUDA events while the context's timers run.
struct PhaseScope {
  nsg_ctx* c;
  int phase;
  cudaEvent_t a = nullptr;
  PhaseScope(nsg_ctx* cc, int p) : c(cc), phase(p) {
    if (c->timing) {
      cudaEventCreate(&a);
      cudaEventRecord(a, c->stream);
    }
  }
  ~PhaseScope() {
    if (a) {
      cudaEvent_t b = nullptr;
      cudaEventCreate(&b);
      cudaEventRecord(b, c->stream);
      c->phases.push_back({phase, a, b, 0.0});
    }
  }
};
void check_launch(const char* what);
// Make the context's device current on the calling thread (every public entry point
// does this first, so a context created for device k works from any thread).
void bind_device(const nsg_ctx* c);
// Raise a kernel's dynamic shared-memory limit on the current device, never lower it.
// cudaFuncSetAttribute applies to the device current when it is called, and contexts on
// other host threads (or devices) launch the same kernels concurrently with other sizes,
// so the limit is tracked per (device, kernel) and only ever raised.
void ensure_smem_limit(const void* fn, int bytes);

// ---------------------------------------------------------------------------
// kernels (launchers)
// ---------------------------------------------------------------------------
// op: 0 = N, 1 = T, 2 = C (conjugate transpose), 3 = R (conjugate, no transpose)
enum Op { OP_N = 0, OP_T = 1, OP_C = 2, OP_R = 3 };

struct GemmArgs {
  int dtype;
  int64_t M, N, K;
  const void* A; int64_t lda; int64_t strideA; int opA;
  const void* B; int64_t ldb; int64_t strideB; int opB;
  void* C; int64_t ldc; int64_t strideC;
  int64_t batch;
  double alpha_re = 1.0, alpha_im = 0.0, beta_re = 0.0, beta_im = 0.0;
};
// dispatches by the context's precision mode and shape
void gemm(nsg_ctx* c, const GemmArgs& g);
void gemm_f64_simt(nsg_ctx* c, const GemmArgs& g);
void gemm_accurate(nsg_ctx* c, const GemmArgs& g);  // FP64-level: Ozaki or FP64 cores
bool gemm_split_tc(nsg_ctx* c, const GemmArgs& g);  // TF32x3; false if not applicable
bool gemm_ozaki_tc(nsg_ctx* c, const GemmArgs& g, int slices = 6);  // BF16 6 or 8 slices; false if not applicable

void permute(nsg_ctx* c, const nsg_tensor* x, const int* perm, bool conj, nsg_tensor* out);
void axpby(nsg_ctx* c, int dtype, int64_t n, double ar, double ai, const void* x, double br,
           double bi, void* y);
// out[j] = <v_j, w> for j < nv (complex: 2 doubles each), written to host buffer
void multi_dot(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const void* w,
               double* host_out);
// w += sum_j coef_j v_j (coef complex pairs)
void multi_axpy(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v,
                const double* coef, void* w);
// device-resident forms (no host synchronisation): the dot products land in out_dev
// (2 doubles each); the coefficients / the sum of squares are read from device memory
void multi_dot_dev(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const void* w, double* out_dev);
void multi_axpy_devcoef(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const double* coef_dev,
                        double sign, void* w);
// y = x / sqrt(s) (mode 0) or y -= sqrt(s) x (mode 1), s = s_dev[0]
void axpby_devscalar(nsg_ctx* c, int dtype, int64_t n, const double* s_dev, int mode, const void* x, void* y);
double norm2(nsg_ctx* c, int dtype, int64_t n, const void* x);
double amax(nsg_ctx* c, int dtype, int64_t n, const void* x);  // max |component|
void scale(nsg_ctx* c, int dtype, int64_t n, double ar, double ai, void* x);
void copy_columns(nsg_ctx* c, int dtype, int64_t rows, int64_t ncols, const void* src,
                  int64_t lds, const int* d_colidx, void* dst, int64_t ldd);
void copy_rows(nsg_ctx* c, int dtype, int64_t nrows_out, int64_t ncols, const void* src,
               int64_t lds, void* dst, int64_t ldd);
void row_norms2(nsg_ctx* c, int dtype, int64_t rows, int64_t cols, const void* A, int64_t lda,
                double* out_dev);

// Hermitian eigensolver (tridiagonalisation + divide and conquer + back-transformation).
// A (n x n) is consumed.  `pick` receives the eigenvalues in ascending order and returns
// the indices whose eigenvectors are wanted, after pointing *Z / *ldz at the output.
using PickFn = std::function<std::vector<int>(const std::vector<double>&, void** Z, int64_t* ldz)>;
void syevd_dc(nsg_ctx* c, int dtype, int n, void* A, std::vector<double>& w_host, const PickFn& pick);

// host helpers
void tridiag_eig(int n, const double* alpha, const double* beta, double* evals, double* evecs);

}  // namespace nsg

// extern "C" guard helper
#define NSG_API_BEGIN(ctx) try { ::nsg::bind_device(ctx);
#define NSG_API_END(ctx)                                                   \
  ::nsg::check_device_flag(ctx);                                           \
  }                                                                        \
  catch (const ::nsg::Error& e) {                                          \
    if (ctx) (ctx)->err = e.what();                                        \
    return e.code;                                                         \
  }                                                                        \
  catch (const std::exception& e) {                                        \
    if (ctx) (ctx)->err = e.what();                                        \
    return NSG_ERR_INVALID;                                                \
  }                                                                        \
  return NSG_OK;
