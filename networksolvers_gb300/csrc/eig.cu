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

// D <- G - I (k x k): the deviation of a Gram matrix from the identity
template <typename T>
__global__ void sub_identity_kernel(T* G, int64_t k) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < k; i += int64_t(gridDim.x) * blockDim.x) {
    if constexpr (sizeof(T) == 8)
      G[i * k + i] -= 1.0;
    else
      G[i * k + i].x -= 1.0;
  }
}

// D <- I - D / 2 with D = G - I: the first-order inverse square root (3 I - G) / 2 of a
// Gram matrix that is the identity up to small terms (symmetric re-orthogonalisation)
template <typename T>
__global__ void newton_step_kernel(T* D, int64_t k) {
  const int64_t tot = k * k;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot; e += int64_t(gridDim.x) * blockDim.x) {
    const bool diag = (e % k) == (e / k);
    if constexpr (sizeof(T) == 8) {
      D[e] = (diag ? 1.0 : 0.0) - 0.5 * D[e];
    } else {
      D[e].x = (diag ? 1.0 : 0.0) - 0.5 * D[e].x;
      D[e].y = -0.5 * D[e].y;
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
// = V S^2 V^H; the spectrum and the truncation rule are those of M M^H (same non-zero
// eigenvalues), C = U^H M as in the square route.  U = M V_k S_k^{-1}, in two parts:
//  * resolved columns (s_i^2 > 1e-11 s_max^2): accurate up to rotations among nearby
//    small singular directions (relative size eps s_max^2 / gap); symmetric
//    re-orthogonalisation U <- U (3 I - U^H U) / 2, repeated until U^H U = I to 1e-14;
//  * the tail below (singular values the Gram matrix resolves only to its rounding):
//    these columns span the right small-singular space but as an ill-conditioned basis;
//    they are projected off the resolved columns twice and orthonormalised through the
//    eigen-decomposition of their own Gram matrix (W <- W E D^-1/2 E^H), then the whole U
//    gets the same re-orthogonalisation.
// Returns false, having allocated nothing that outlives it, when the tail is exactly rank
// deficient, a kept weight is not positive, or the tail's eigenproblem would make the
// route dearer than M M^H (tail + ncol > m): the caller then takes the M M^H route.
static bool factorize_right(nsg_ctx* c, nsg_tensor* M, int64_t m, int64_t ncol, const std::vector<int64_t>& ldims,
                            const std::vector<int64_t>& rdims, double sc, double cutoff, int64_t maxdim,
                            int64_t mindim, nsg_tensor** Uo, nsg_tensor** Co, int64_t* ko, double* erro,
                            std::vector<double>& P) {
  const int dt = M->dtype;
  const size_t eb = elem_bytes(dt);
  const int64_t n = ncol;
  auto mm = [&](int64_t M_, int64_t N_, int64_t K_, const void* A, int64_t lda, int opA, const void* B, int64_t ldb,
                int opB, void* C, int64_t ldc, double alpha, double beta) {
    GemmArgs g;
    g.dtype = dt;
    g.M = M_;
    g.N = N_;
    g.K = K_;
    g.A = A;
    g.lda = lda;
    g.opA = opA;
    g.B = B;
    g.ldb = ldb;
    g.opB = opB;
    g.C = C;
    g.ldc = ldc;
    g.batch = 1;
    g.strideA = g.strideB = g.strideC = 0;
    g.alpha_re = alpha;
    g.beta_re = beta;
    gemm_accurate(c, g);
  };
  void* G = dalloc(c, eb * n * n);
  mm(n, n, m, M->data, m, OP_C, M->data, m, OP_N, G, n, 1.0, 0.0);  // FP64-level: fixes the truncation
  int64_t k = 0, kr = 0;
  double err = 0.0;
  bool ok = true;
  void* V = nullptr;
  size_t vbytes = 0;
  std::vector<double> w;
  PickFn pick = [&](const std::vector<double>& wa, void** Z, int64_t* ldz) {
    P.assign(wa.rbegin(), wa.rend());
    k = truncate_rule(P, n, cutoff, maxdim, mindim, &err);
    kr = 0;
    while (kr < k && P[kr] > 1e-11 * P[0]) ++kr;
    ok = P[0] > 0.0 && P[k - 1] > 0.0 && (k - kr) + n <= m;
    if (!ok) return std::vector<int>();
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
  // U = M V_k S_k^{-1}
  std::vector<int64_t> udims = ldims;
  udims.push_back(k);
  nsg_tensor* Ut = new_tensor(c, dt, int(udims.size()), udims.data(), false);
  mm(m, k, n, M->data, m, OP_N, V, n, OP_N, Ut->data, m, 1.0, 0.0);
  dfree(c, V, vbytes);
  const int gsms = int(c->num_sms) * 8;
  auto col_scale = [&](void* Y, int64_t rows, int64_t cols, const double* f_dev) {
    const int gb = int(std::min<int64_t>((rows * cols + 255) / 256, gsms));
    if (dt == NSG_C128)
      col_scale_kernel<double2><<<gb, 256, 0, c->stream>>>((double2*)Y, rows, cols, f_dev);
    else
      col_scale_kernel<double><<<gb, 256, 0, c->stream>>>((double*)Y, rows, cols, f_dev);
    count_launch(c);
  };
  {
    std::vector<double> inv(k);
    for (int64_t i = 0; i < k; ++i) inv[i] = 1.0 / std::sqrt(P[i]);
    DevBuf1 f(c, sizeof(double) * k);
    NSG_CUDA(cudaMemcpyAsync(f.p, inv.data(), sizeof(double) * k, cudaMemcpyHostToDevice, c->stream));
    col_scale(Ut->data, m, k, (const double*)f.p);
    NSG_CUDA(cudaStreamSynchronize(c->stream));  // inv leaves scope
  }
  char* U = (char*)Ut->data;
  const int64_t kt = k - kr;
  void* Y2 = dalloc(c, eb * m * k);
  void* Gk = dalloc(c, eb * k * k);
  // symmetric re-orthogonalisation of the first kk columns until U^H U = I to the
  // rounding of the Gram product (or until a step stops gaining); false when U^H U is too
  // far from I for the iteration to converge, or it ends above 1e-13
  const double floor_tol = std::max(1e-14, 8.0 * 2.220446049250313e-16 * std::sqrt(double(m)));
  auto lowdin = [&](int64_t kk) -> bool {
    double prev = 1.0;
    for (int it = 0; it < 6; ++it) {
      mm(kk, kk, m, U, m, OP_C, U, m, OP_N, Gk, kk, 1.0, 0.0);
      const int gb = int(std::min<int64_t>((kk * kk + 255) / 256, gsms));
      if (dt == NSG_C128)
        sub_identity_kernel<double2><<<gb, 256, 0, c->stream>>>((double2*)Gk, kk);
      else
        sub_identity_kernel<double><<<gb, 256, 0, c->stream>>>((double*)Gk, kk);
      count_launch(c);
      const double dev = amax(c, dt, kk * kk, Gk);
      if (!(dev < 0.1 / std::sqrt(double(kk)))) return false;
      if (dev < floor_tol) return true;
      if (dev > 0.1 * prev) return dev < 1e-13;  // at the rounding floor
      prev = dev;
      if (dt == NSG_C128)
        newton_step_kernel<double2><<<gb, 256, 0, c->stream>>>((double2*)Gk, kk);
      else
        newton_step_kernel<double><<<gb, 256, 0, c->stream>>>((double*)Gk, kk);
      count_launch(c);
      mm(m, kk, kk, U, m, OP_N, Gk, kk, OP_N, Y2, m, 1.0, 0.0);
      NSG_CUDA(cudaMemcpyAsync(U, Y2, eb * m * kk, cudaMemcpyDeviceToDevice, c->stream));
    }
    return prev < 1e-13;
  };
  bool good = lowdin(kr);
  if (good && kt > 0) {
    void* W = U + eb * m * kr;
    // project the tail off the resolved columns (twice), then orthonormalise it
    for (int pass = 0; pass < 2; ++pass) {
      mm(kr, kt, m, U, m, OP_C, W, m, OP_N, Gk, kr, 1.0, 0.0);
      mm(m, kt, kr, U, m, OP_N, Gk, kr, OP_N, W, m, -1.0, 1.0);
    }
    void* Gt = dalloc(c, eb * kt * kt);
    mm(kt, kt, m, W, m, OP_C, W, m, OP_N, Gt, kt, 1.0, 0.0);
    void* E = dalloc(c, eb * kt * kt);
    std::vector<double> wt;
    PickFn all = [&](const std::vector<double>&, void** Z, int64_t* ldz) {
      *Z = E;
      *ldz = kt;
      std::vector<int> cols(kt);
      std::iota(cols.begin(), cols.end(), 0);
      return cols;
    };
    try {
      syevd_dc(c, dt, int(kt), Gt, wt, all);
    } catch (...) {
      dfree(c, Gt, eb * kt * kt);
      dfree(c, E, eb * kt * kt);
      dfree(c, Y2, eb * m * k);
      dfree(c, Gk, eb * k * k);
      free_tensor(c, Ut);
      throw;
    }
    dfree(c, Gt, eb * kt * kt);
    good = wt[0] > 1e-13 * wt[kt - 1] && wt[kt - 1] > 0.0;
    if (good) {
      std::vector<double> rs(kt);
      for (int64_t i = 0; i < kt; ++i) rs[i] = 1.0 / std::sqrt(wt[i]);
      DevBuf1 f(c, sizeof(double) * kt);
      NSG_CUDA(cudaMemcpyAsync(f.p, rs.data(), sizeof(double) * kt, cudaMemcpyHostToDevice, c->stream));
      void* F = Y2;  // E D^-1/2, then X = F E^H, then W X (scratch regions do not overlap)
      NSG_CUDA(cudaMemcpyAsync(F, E, eb * kt * kt, cudaMemcpyDeviceToDevice, c->stream));
      col_scale(F, kt, kt, (const double*)f.p);
      mm(kt, kt, kt, F, kt, OP_N, E, kt, OP_C, Gk, kt, 1.0, 0.0);
      mm(m, kt, kt, W, m, OP_N, Gk, kt, OP_N, Y2, m, 1.0, 0.0);
      NSG_CUDA(cudaMemcpyAsync(W, Y2, eb * m * kt, cudaMemcpyDeviceToDevice, c->stream));
      NSG_CUDA(cudaStreamSynchronize(c->stream));  // rs leaves scope
      mm(kr, kt, m, U, m, OP_C, W, m, OP_N, Gk, kr, 1.0, 0.0);
      mm(m, kt, kr, U, m, OP_N, Gk, kr, OP_N, W, m, -1.0, 1.0);
      good = lowdin(k);
    }
    dfree(c, E, eb * kt * kt);
  }
  dfree(c, Y2, eb * m * k);
  dfree(c, Gk, eb * k * k);
  check_launch("factorize (tall)");
  if (!good) {
    free_tensor(c, Ut);
    return false;
  }
  // C = U^H M
  std::vector<int64_t> cdims;
  cdims.push_back(k);
  for (auto d : rdims) cdims.push_back(d);
  nsg_tensor* Ct = new_tensor(c, dt, int(cdims.size()), cdims.data(), false);
  mm(k, ncol, m, Ut->data, m, OP_C, M->data, m, OP_N, Ct->data, k, sc, 0.0);
  *Uo = Ut;
  *Co = Ct;
  *ko = k;
  *erro = err;
  return true;
}


static int factorize_impl(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, double cutoff,
                          int64_t maxdim, int64_t mindim, nsg_tensor** U, nsg_tensor** C, int64_t* newdim,
                          double* truncerr, double* spectrum, int64_t spectrum_cap, nsg_tensor** Uperp = nullptr) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && T && U && C, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(n_left >= 1 && n_left < T->rank, NSG_ERR_INVALID, "factorize: need left and right axes");
  if (Uperp) *Uperp = nullptr;
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
  // The narrow side's Gram matrix is tried unless the call keeps everything (cutoff 0 and
  // no maxdim below the narrow side, as a QR does): then the kept weights reach the Gram
  // matrix's rounding, a rank-deficient M makes the route give up after its eigensolver,
  // and M M^H is taken directly.
  const bool tall_may_pass = cutoff > 0.0 || (maxdim > 0 && maxdim < ncol);
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
  // with Uperp requested, every eigenvector is back-transformed (kept ones first): the
  // discarded ones are an orthonormal basis of the complement of U's columns
  void* Zall = nullptr;
  size_t zbytes = 0;
  PickFn pick = [&](const std::vector<double>& wa, void** Z, int64_t* ldz) {
    // descending spectrum
    P.assign(wa.rbegin(), wa.rend());
    k = truncate_rule(P, origm, cutoff, maxdim, mindim, &err);
    std::vector<int64_t> udims = ldims;
    udims.push_back(k);
    Ut = new_tensor(c, dt, int(udims.size()), udims.data(), false);
    const int64_t ncols = (Uperp && k < m) ? m : k;
    if (ncols > k) {
      zbytes = eb * size_t(m) * size_t(m);
      Zall = dalloc(c, zbytes);
    }
    *Z = Zall ? Zall : Ut->data;
    *ldz = m;
    std::vector<int> cols(ncols);
    for (int64_t i = 0; i < ncols; ++i) cols[i] = int(m - 1 - i);
    return cols;
  };
  try {
    syevd_dc(c, dt, int(m), G, w, pick);
  } catch (...) {
    dfree(c, G, eb * m * m);
    if (Ut) free_tensor(c, Ut);
    if (Zall) dfree(c, Zall, zbytes);
    if (owned) free_tensor(c, M);
    throw;
  }
  dfree(c, G, eb * m * m);
  if (Zall) {
    std::vector<int64_t> pdims = ldims;
    pdims.push_back(m - k);
    nsg_tensor* Qp = new_tensor(c, dt, int(pdims.size()), pdims.data(), false);
    NSG_CUDA(cudaMemcpyAsync(Ut->data, Zall, eb * size_t(m) * size_t(k), cudaMemcpyDeviceToDevice, c->stream));
    NSG_CUDA(cudaMemcpyAsync(Qp->data, (char*)Zall + eb * size_t(m) * size_t(k), eb * size_t(m) * size_t(m - k),
                             cudaMemcpyDeviceToDevice, c->stream));
    dfree(c, Zall, zbytes);
    *Uperp = Qp;
  }
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

int nsg_factorize_complement(nsg_ctx* c, const nsg_tensor* T, const int* left_axes, int n_left, double cutoff,
                             int64_t maxdim, int64_t mindim, nsg_tensor** U, nsg_tensor** C, nsg_tensor** Uperp,
                             int64_t* newdim, double* truncerr) {
  if (!Uperp) return factorize_impl(c, T, left_axes, n_left, cutoff, maxdim, mindim, U, C, newdim, truncerr,
                                    nullptr, 0);
  return factorize_impl(c, T, left_axes, n_left, cutoff, maxdim, mindim, U, C, newdim, truncerr, nullptr, 0, Uperp);
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
