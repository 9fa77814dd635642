// Truncated factorizations of the inserter and the subspace expansion:
//   it.factorize(local, indsTe; cutoff, maxdim, mindim)   inserter.jl:23
//   qr(...)                                               extracter.jl:6, applyexp.jl:37
//   eigen(rho; trunc..., ishermitian=true)                 subspace/densitymatrix.jl:53
//
// The SVD of the matricised tensor M (m x n) goes through a Hermitian Gram matrix.
// m <= n: G = M M^H = Z diag(lambda) Z^H gives the left singular vectors U = Z and
// sigma^2 = lambda, and C = U^H M = S V^H is the right factor that `factorize` with
// ortho="left" stores (U -> psi[v1], C -> psi[v2]).  m > n: the narrow side's Gram
// matrix M^H M = V S^2 V^H, U = M V S^-1 re-orthogonalised, C = U^H M.  The Hermitian
// eigenproblems go to the tridiagonalisation + divide-and-conquer solver (syevd.cu).
// Every product here is FP64-level: the FP64 cores, or in the split precision the
// eight-slice Ozaki form (real data), whose error is at the FP64 rounding level of the
// operand scales; the Gram matrix stays exactly symmetric in both (same slices on both
// sides, exact integer partial sums).
//
// Truncation rule (NDTensors, restated): spectrum P = lambda sorted descending,
// negative tail zeroed; cut to maxdim; then drop from the end while
// (discarded + P[n] < cutoff * sum(P)) and n > mindim.
#include "nsg_internal.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace nsg {

namespace {

// NDTensors truncation rule; returns kept count and relative discarded weight.
int64_t truncate_rule(std::vector<double> P, int64_t origm, double cutoff, int64_t maxdim, int64_t mindim,
                      double* truncerr) {
  P.resize(origm);
  for (int64_t n = origm - 1; n >= 0; --n) {
    if (P[n] >= 0) break;
    P[n] = 0.0;
  }
  int64_t md = (maxdim <= 0) ? origm : std::min<int64_t>(maxdim, origm);
  int64_t n = origm;
  double err = 0.0;
  while (n > md) {
    err += P[n - 1];
    --n;
  }
  double scale = 0.0;
  for (double x : P) scale += x;
  if (scale == 0.0) scale = 1.0;
  while (n > mindim && err + P[n - 1] < cutoff * scale) {
    err += P[n - 1];
    --n;
  }
  if (n < 1) n = 1;
  *truncerr = err / scale;
  return n;
}

// permute T so that the listed axes come first; returns matrix dims
nsg_tensor* matricize(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, int64_t* m, int64_t* ncol,
                      std::vector<int64_t>& ldims, std::vector<int64_t>& rdims, bool* owned) {
  std::vector<int> perm;
  std::vector<int> used(T->rank, 0);
  for (int k = 0; k < n_left; ++k) {
    NSG_CHECK(left_axes[k] >= 0 && left_axes[k] < T->rank && !used[left_axes[k]], NSG_ERR_INVALID,
              "factorize: bad left axes");
    used[left_axes[k]] = 1;
    perm.push_back(left_axes[k]);
  }
  for (int k = 0; k < T->rank; ++k)
    if (!used[k]) perm.push_back(k);
  *m = 1;
  *ncol = 1;
  ldims.clear();
  rdims.clear();
  for (int k = 0; k < T->rank; ++k) {
    int64_t d = T->dims[perm[k]];
    if (k < n_left) {
      *m *= d;
      ldims.push_back(d);
    } else {
      *ncol *= d;
      rdims.push_back(d);
    }
  }
  bool ident = true;
  for (int k = 0; k < T->rank; ++k) ident &= perm[k] == k;
  if (ident) {
    *owned = false;
    return const_cast<nsg_tensor*>(T);
  }
  int64_t dims[NSG_MAX_RANK];
  for (int k = 0; k < T->rank; ++k) dims[k] = T->dims[perm[k]];
  nsg_tensor* P = new_tensor(c, T->dtype, T->rank, dims, false);
  permute(c, T, perm.data(), false, P);
  *owned = true;
  return P;
}


// Y[:, j] *= f[j]  (column scaling)
template <typename T>
__global__ void col_scale_kernel(T* Y, int64_t rows, int64_t cols, const double* f) {
  const int64_t tot = rows * cols;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot; e += int64_t(gridDim.x) * blockDim.x) {
    const double s = f[e / rows];
    if constexpr (sizeof(T) == 8) {
      Y[e] *= s;
    } else {
      Y[e].x *= s;
      Y[e].y *= s;
    }
  }
}

// G <- 1.5 I - 0.5 G (k x k): the first-order inverse square root of a Gram matrix
// that is the identity up to small terms (symmetric re-orthogonalisation)
template <typename T>
__global__ void half_newton_kernel(T* G, int64_t k) {
  const int64_t tot = k * k;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot; e += int64_t(gridDim.x) * blockDim.x) {
    const bool diag = (e % k) == (e / k);
    if constexpr (sizeof(T) == 8) {
      G[e] = (diag ? 1.5 : 0.0) - 0.5 * G[e];
    } else {
      G[e].x = (diag ? 1.5 : 0.0) - 0.5 * G[e].x;
      G[e].y = -0.5 * G[e].y;
    }
  }
}

}  // namespace

}  // namespace nsg

using namespace nsg;

namespace {
struct DevBuf1 {
  nsg_ctx* c;
  void* p;
  size_t bytes;
  DevBuf1(nsg_ctx* cc, size_t b) : c(cc), p(dalloc(cc, b)), bytes(b) {}
  ~DevBuf1() { dfree(c, p, bytes); }
};
}  // namespace

// Tall M (m > ncol): truncated factorisation from the smaller Gram matrix M^H M
// = V S^2 V^H.  U = M V_k S_k^{-1} carries a relative column error ~ eps s_max / s_k,
// removed by symmetric re-orthogonalisation U <- U (3 I - U^H U) / 2 (each step squares
// it; two steps when eps s_max / s_k > 1e-8); C = U^H M as in the square route.  The
// spectrum and the truncation rule are those of M M^H (same non-zero eigenvalues).
// Returns false, having allocated nothing that outlives it, when s_k^2 <= 1e-11 s_max^2
// (s_k not resolved by the Gram matrix well above its rounding): the caller then takes
// the M M^H route.
static bool factorize_right(nsg_ctx* c, nsg_tensor* M, int64_t m, int64_t ncol, const std::vector<int64_t>& ldims,
                            const std::vector<int64_t>& rdims, double sc, double cutoff, int64_t maxdim,
                            int64_t mindim, nsg_tensor** Uo, nsg_tensor** Co, int64_t* ko, double* erro,
                            std::vector<double>& P) {
  const int dt = M->dtype;
  const size_t eb = elem_bytes(dt);
  const int64_t n = ncol;
  void* G = dalloc(c, eb * n * n);
  GemmArgs g;
  g.dtype = dt;
  g.M = n;
  g.N = n;
  g.K = m;
  g.A = M->data;
  g.lda = m;
  g.opA = OP_C;
  g.B = M->data;
  g.ldb = m;
  g.opB = OP_N;
  g.C = G;
  g.ldc = n;
  g.batch = 1;
  g.strideA = g.strideB = g.strideC = 0;
  gemm_accurate(c, g);  // FP64-level product: the Gram matrix fixes the truncation
  int64_t k = 0;
  double err = 0.0, delta = 0.0;
  bool ok = true;
  void* V = nullptr;
  size_t vbytes = 0;
  std::vector<double> w;
  PickFn pick = [&](const std::vector<double>& wa, void** Z, int64_t* ldz) {
    P.assign(wa.rbegin(), wa.rend());
    k = truncate_rule(P, n, cutoff, maxdim, mindim, &err);
    // the Gram eigenvalues carry ~1e-15 P[0] of rounding: s_k must be resolved well above it
    const double smax = std::sqrt(std::max(P[0], 0.0)), smin = std::sqrt(std::max(P[k - 1], 0.0));
    ok = smax > 0.0 && P[k - 1] > 1e-11 * P[0];
    if (!ok) return std::vector<int>();
    delta = 1e-16 * smax / smin;
    vbytes = eb * size_t(n) * size_t(k);
    V = dalloc(c, vbytes);
    *Z = V;
    *ldz = n;
    std::vector<int> cols(k);
    for (int64_t i = 0; i < k; ++i) cols[i] = int(n - 1 - i);
    return cols;
  };
  try {
    syevd_dc(c, dt, int(n), G, w, pick);
  } catch (...) {
    dfree(c, G, eb * n * n);
    if (V) dfree(c, V, vbytes);
    throw;
  }
  dfree(c, G, eb * n * n);
  if (!ok) return false;
  // Y = M V_k S_k^{-1}
  std::vector<int64_t> udims = ldims;
  udims.push_back(k);
  nsg_tensor* Ut = new_tensor(c, dt, int(udims.size()), udims.data(), false);
  GemmArgs y;
  y.dtype = dt;
  y.M = m;
  y.N = k;
  y.K = n;
  y.A = M->data;
  y.lda = m;
  y.opA = OP_N;
  y.B = V;
  y.ldb = n;
  y.opB = OP_N;
  y.C = Ut->data;
  y.ldc = m;
  y.batch = 1;
  y.strideA = y.strideB = y.strideC = 0;
  gemm_accurate(c, y);
  dfree(c, V, vbytes);
  {
    std::vector<double> inv(k);
    for (int64_t i = 0; i < k; ++i) inv[i] = 1.0 / std::sqrt(P[i]);
    DevBuf1 f(c, sizeof(double) * k);
    NSG_CUDA(cudaMemcpyAsync(f.p, inv.data(), sizeof(double) * k, cudaMemcpyHostToDevice, c->stream));
    const int gb = int(std::min<int64_t>((m * k + 255) / 256, int64_t(c->num_sms) * 8));
    if (dt == NSG_C128)
      col_scale_kernel<double2><<<gb, 256, 0, c->stream>>>((double2*)Ut->data, m, k, (const double*)f.p);
    else
      col_scale_kernel<double><<<gb, 256, 0, c->stream>>>((double*)Ut->data, m, k, (const double*)f.p);
    count_launch(c);
    NSG_CUDA(cudaStreamSynchronize(c->stream));  // inv leaves scope
  }
  // symmetric re-orthogonalisation
  const int iters = delta > 1e-8 ? 2 : 1;
  nsg_tensor* Y2 = new_tensor(c, dt, int(udims.size()), udims.data(), false);
  void* Gk = dalloc(c, eb * k * k);
  for (int it = 0; it < iters; ++it) {
    GemmArgs q = y;
    q.M = k;
    q.N = k;
    q.K = m;
    q.A = Ut->data;
    q.lda = m;
    q.opA = OP_C;
    q.B = Ut->data;
    q.ldb = m;
    q.opB = OP_N;
    q.C = Gk;
    q.ldc = k;
    gemm_accurate(c, q);
    const int gb = int(std::min<int64_t>((k * k + 255) / 256, int64_t(c->num_sms) * 8));
    if (dt == NSG_C128)
      half_newton_kernel<double2><<<gb, 256, 0, c->stream>>>((double2*)Gk, k);
    else
      half_newton_kernel<double><<<gb, 256, 0, c->stream>>>((double*)Gk, k);
    count_launch(c);
    GemmArgs r = y;
    r.M = m;
    r.N = k;
    r.K = k;
    r.A = Ut->data;
    r.lda = m;
    r.opA = OP_N;
    r.B = Gk;
    r.ldb = k;
    r.opB = OP_N;
    r.C = Y2->data;
    r.ldc = m;
    gemm_accurate(c, r);
    std::swap(Ut, Y2);
  }
  dfree(c, Gk, eb * k * k);
  free_tensor(c, Y2);
  check_launch("factorize (tall)");
  // C = U^H M
  std::vector<int64_t> cdims;
  cdims.push_back(k);
  for (auto d : rdims) cdims.push_back(d);
  nsg_tensor* Ct = new_tensor(c, dt, int(cdims.size()), cdims.data(), false);
  GemmArgs h = y;
  h.M = k;
  h.N = ncol;
  h.K = m;
  h.A = Ut->data;
  h.lda = m;
  h.opA = OP_C;
  h.B = M->data;
  h.ldb = m;
  h.opB = OP_N;
  h.C = Ct->data;
  h.ldc = k;
  h.alpha_re = sc;
  gemm_accurate(c, h);
  *Uo = Ut;
  *Co = Ct;
  *ko = k;
  *erro = err;
  return true;
}


static int factorize_impl(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, double cutoff,
                          int64_t maxdim, int64_t mindim, nsg_tensor** U, nsg_tensor** C, int64_t* newdim,
                          double* truncerr, double* spectrum, int64_t spectrum_cap) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && T && U && C, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(n_left >= 1 && n_left < T->rank, NSG_ERR_INVALID, "factorize: need left and right axes");
  int64_t m, ncol;
  std::vector<int64_t> ldims, rdims;
  bool owned = false;
  nsg_tensor* M = matricize(c, T, left_axes, n_left, &m, &ncol, ldims, rdims, &owned);
  const int dt = T->dtype;
  const size_t eb = elem_bytes(dt);
  NSG_CHECK(m <= (1 << 16), NSG_ERR_UNSUPPORTED, "factorize: row space above 65536");
  // The Gram route squares magnitudes: bring the entries to O(1) first (tensors of
  // un-normalised networks reach 1e150 and beyond) and scale C back at the end.
  double mx = amax(c, dt, M->size, M->data);
  NSG_CHECK(std::isfinite(mx), NSG_ERR_NONFINITE, "factorize: non-finite input");
  double sc = 1.0;
  if (mx > 0 && (mx > 1e50 || mx < 1e-50)) {
    sc = mx;
    if (!owned) {
      nsg_tensor* Mc = new_tensor(c, M->dtype, M->rank, M->dims, false);
      NSG_CUDA(cudaMemcpyAsync(Mc->data, M->data, M->bytes, cudaMemcpyDeviceToDevice, c->stream));
      M = Mc;
      owned = true;
    }
    scale(c, dt, M->size, 1.0 / sc, 0.0, M->data);
  }
  // The tall route is kept only when its smallest kept sigma^2 lies above 1e-11 of the
  // largest (checked once the spectrum is known, before any eigenvector is formed).  A
  // truncation that only the cutoff limits keeps weights down to ~cutoff / (discarded
  // count) of the total, so with cutoff < 1e-10 and no maxdim below the narrow side the
  // check fails on practically every spectrum: the attempt (Gram matrix, tridiagonal
  // reduction and divide and conquer of the narrow side) is then skipped.
  const bool tall_may_pass = cutoff >= 1e-10 || (maxdim > 0 && maxdim < ncol);
  if (ncol < m && ncol >= 16 && tall_may_pass) {
    std::vector<double> Pr;
    nsg_tensor *Ur = nullptr, *Cr = nullptr;
    int64_t kr = 0;
    double er = 0.0;
    bool done;
    try {
      done = factorize_right(c, M, m, ncol, ldims, rdims, sc, cutoff, maxdim, mindim, &Ur, &Cr, &kr, &er, Pr);
    } catch (...) {
      if (owned) free_tensor(c, M);
      throw;
    }
    if (done) {
      if (owned) free_tensor(c, M);
      if (spectrum)
        for (int64_t i = 0; i < std::min<int64_t>(spectrum_cap, ncol); ++i)
          spectrum[i] = i < int64_t(Pr.size()) ? std::max(Pr[i], 0.0) * sc * sc : 0.0;
      *U = Ur;
      *C = Cr;
      if (newdim) *newdim = kr;
      if (truncerr) *truncerr = er;
      check_device_flag(c);
      return NSG_OK;
    }
  }
  // G = M M^H (FP64-level product in every precision mode: the Gram matrix fixes the truncation)
  void* G = dalloc(c, eb * m * m);
  GemmArgs g;
  g.dtype = dt;
  g.M = m;
  g.N = m;
  g.K = ncol;
  g.A = M->data;
  g.lda = m;
  g.opA = OP_N;
  g.B = M->data;
  g.ldb = m;
  g.opB = OP_C;
  g.C = G;
  g.ldc = m;
  g.batch = 1;
  g.strideA = g.strideB = g.strideC = 0;
  gemm_accurate(c, g);
  const int64_t origm = std::min(m, ncol);
  double err = 0.0;
  int64_t k = 0;
  nsg_tensor* Ut = nullptr;
  std::vector<double> P;
  std::vector<double> w;
  PickFn pick = [&](const std::vector<double>& wa, void** Z, int64_t* ldz) {
    // descending spectrum
    P.assign(wa.rbegin(), wa.rend());
    k = truncate_rule(P, origm, cutoff, maxdim, mindim, &err);
    std::vector<int64_t> udims = ldims;
    udims.push_back(k);
    Ut = new_tensor(c, dt, int(udims.size()), udims.data(), false);
    *Z = Ut->data;
    *ldz = m;
    std::vector<int> cols(k);
    for (int64_t i = 0; i < k; ++i) cols[i] = int(m - 1 - i);
    return cols;
  };
  try {
    syevd_dc(c, dt, int(m), G, w, pick);
  } catch (...) {
    dfree(c, G, eb * m * m);
    if (Ut) free_tensor(c, Ut);
    if (owned) free_tensor(c, M);
    throw;
  }
  dfree(c, G, eb * m * m);
  // C = U^H M
  std::vector<int64_t> cdims;
  cdims.push_back(k);
  for (auto d : rdims) cdims.push_back(d);
  nsg_tensor* Ct = new_tensor(c, dt, int(cdims.size()), cdims.data(), false);
  GemmArgs h;
  h.dtype = dt;
  h.M = k;
  h.N = ncol;
  h.K = m;
  h.A = Ut->data;
  h.lda = m;
  h.opA = OP_C;
  h.B = M->data;
  h.ldb = m;
  h.opB = OP_N;
  h.C = Ct->data;
  h.ldc = k;
  h.batch = 1;
  h.strideA = h.strideB = h.strideC = 0;
  h.alpha_re = sc;
  gemm_accurate(c, h);  // FP64-level: C carries the small singular directions of the next region
  if (owned) free_tensor(c, M);
  if (spectrum)
    for (int64_t i = 0; i < std::min<int64_t>(spectrum_cap, origm); ++i)
      spectrum[i] = i < int64_t(P.size()) ? std::max(P[i], 0.0) * sc * sc : 0.0;
  *U = Ut;
  *C = Ct;
  if (newdim) *newdim = k;
  if (truncerr) *truncerr = err;
  NSG_API_END(c)
}

extern "C" {

int nsg_factorize(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, double cutoff, int64_t maxdim,
                  int64_t mindim, nsg_tensor** U, nsg_tensor** C, int64_t* newdim, double* truncerr,
                  double* spectrum, int64_t spectrum_cap) {
  return factorize_impl(c, T, left_axes, n_left, cutoff, maxdim, mindim, U, C, newdim, truncerr, spectrum,
                        spectrum_cap);
}

int nsg_qr(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, nsg_tensor** Q, nsg_tensor** R) {
  int64_t k;
  double err;
  return factorize_impl(c, T, left_axes, n_left, 0.0, 0, 1, Q, R, &k, &err, nullptr, 0);
}

int nsg_eigh(nsg_ctx* c, const nsg_tensor* rho, const int* row_axes, int n_row, double cutoff, int64_t maxdim,
             int64_t mindim, nsg_tensor** U, double* evals, int64_t evals_cap, int64_t* newdim, double* truncerr) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && rho && U, NSG_ERR_INVALID, "null argument");
  int64_t m, ncol;
  std::vector<int64_t> ldims, rdims;
  bool owned = false;
  nsg_tensor* M = matricize(c, rho, row_axes, n_row, &m, &ncol, ldims, rdims, &owned);
  NSG_CHECK(m == ncol, NSG_ERR_INVALID, "eigh: row and column spaces differ in size");
  const int dt = rho->dtype;
  const size_t eb = elem_bytes(dt);
  void* A = dalloc(c, eb * m * m);
  NSG_CUDA(cudaMemcpyAsync(A, M->data, eb * m * m, cudaMemcpyDeviceToDevice, c->stream));
  if (owned) free_tensor(c, M);
  double err = 0.0;
  int64_t k = 0;
  nsg_tensor* Ut = nullptr;
  std::vector<double> P, w;
  PickFn pick = [&](const std::vector<double>& wa, void** Z, int64_t* ldz) {
    P.assign(wa.rbegin(), wa.rend());
    k = truncate_rule(P, m, cutoff, maxdim, mindim, &err);
    std::vector<int64_t> udims = rdims;
    udims.push_back(k);
    Ut = new_tensor(c, dt, int(udims.size()), udims.data(), false);
    *Z = Ut->data;
    *ldz = m;
    std::vector<int> cols(k);
    for (int64_t i = 0; i < k; ++i) cols[i] = int(m - 1 - i);
    return cols;
  };
  try {
    syevd_dc(c, dt, int(m), A, w, pick);
  } catch (...) {
    dfree(c, A, eb * m * m);
    if (Ut) free_tensor(c, Ut);
    throw;
  }
  dfree(c, A, eb * m * m);
  if (evals)
    for (int64_t i = 0; i < std::min(evals_cap, k); ++i) evals[i] = P[i];
  *U = Ut;
  if (newdim) *newdim = k;
  if (truncerr) *truncerr = err;
  NSG_API_END(c)
}

}  // extern "C"
