// Local solvers of local_solvers/*.jl, with every Krylov vector resident on the
// device.  Only the scalars of the recurrence (alpha, beta, projection
// coefficients) come back to the host, where the k x k tridiagonal problems
// (k <= krylovdim) are solved in FP64.
//
//  * nsg_eigsolve      — KrylovKit `eigsolve(..., :SR; krylovdim, maxiter, tol)` as
//                        called by local_solvers/eigsolve.jl:16-27 (Lanczos).
//  * nsg_exponentiate  — KrylovKit `exponentiate(A, t, x; krylovdim, tol, maxiter,
//                        eager)`, local_solvers/exponentiate.jl:16-27.
//  * nsg_runge_kutta   — runge_kutta.jl:2-25.
//
// Lanczos step (shared by both Krylov solvers): w = A v_j - beta_{j-1} v_{j-1},
// then two full classical Gram-Schmidt passes against v_0..v_j; alpha_j is the sum
// of the two projections on v_j and beta_j = ||w||.
#include "nsg_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>

namespace nsg {
void linmap_apply(nsg_ctx* c, nsg_linmap* m, const nsg_tensor* x, nsg_tensor* y);

// Dense symmetric eigensolver for small host matrices (cyclic Jacobi).
// A: n x n column-major (destroyed), w: eigenvalues ascending, V: eigenvectors.
static void sym_eig_small(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& V) {
  V.assign(size_t(n) * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + size_t(n) * i] = 1.0;
  auto a = [&](int i, int j) -> double& { return A[i + size_t(n) * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        tot += a(i, j) * a(i, j);
        if (i != j) off += a(i, j) * a(i, j);
      }
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        double theta = (a(q, q) - a(p, p)) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < n; ++k) {  // columns
          double akp = a(k, p), akq = a(k, q);
          a(k, p) = cs * akp - sn * akq;
          a(k, q) = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows
          double apk = a(p, k), aqk = a(q, k);
          a(p, k) = cs * apk - sn * aqk;
          a(q, k) = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k + size_t(n) * p], vkq = V[k + size_t(n) * q];
          V[k + size_t(n) * p] = cs * vkp - sn * vkq;
          V[k + size_t(n) * q] = sn * vkp + cs * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  std::vector<double> Vs(size_t(n) * n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    w[k] = a(idx[k], idx[k]);
    for (int i = 0; i < n; ++i) Vs[i + size_t(n) * k] = V[i + size_t(n) * idx[k]];
  }
  V.swap(Vs);
}

void tridiag_eig(int n, const double* alpha, const double* beta, double* evals, double* evecs) {
  std::vector<double> A(size_t(n) * n, 0.0), w, V;
  for (int i = 0; i < n; ++i) {
    A[i + size_t(n) * i] = alpha[i];
    if (i + 1 < n) A[i + size_t(n) * (i + 1)] = A[(i + 1) + size_t(n) * i] = beta[i];
  }
  sym_eig_small(n, A, w, V);
  for (int i = 0; i < n; ++i) evals[i] = w[i];
  for (size_t i = 0; i < size_t(n) * n; ++i) evecs[i] = V[i];
}

// exp(A) of a small complex k x k matrix (column-major): scaling and squaring with a
// degree-18 Taylor polynomial on A / 2^s, ||A / 2^s||_1 <= 1/2.  Tiny entries (the
// Krylov error corner) keep their relative accuracy.
static std::vector<std::complex<double>> expm_small(int k, const std::vector<std::complex<double>>& A) {
  using cd = std::complex<double>;
  double nrm = 0.0;
  for (int j = 0; j < k; ++j) {
    double c = 0.0;
    for (int i = 0; i < k; ++i) c += std::abs(A[i + size_t(k) * j]);
    nrm = std::max(nrm, c);
  }
  int s = nrm <= 0.5 ? 0 : int(std::ceil(std::log2(nrm / 0.5)));
  double sc = std::ldexp(1.0, -s);
  std::vector<cd> X(A.size()), E(A.size(), cd(0, 0)), term(A.size(), cd(0, 0)), tmp(A.size());
  for (size_t i = 0; i < A.size(); ++i) X[i] = A[i] * sc;
  for (int i = 0; i < k; ++i) E[i + size_t(k) * i] = term[i + size_t(k) * i] = cd(1, 0);
  auto matmul = [&](const std::vector<cd>& P, const std::vector<cd>& Q, std::vector<cd>& R) {
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) {
        cd acc(0, 0);
        for (int l = 0; l < k; ++l) acc += P[i + size_t(k) * l] * Q[l + size_t(k) * j];
        R[i + size_t(k) * j] = acc;
      }
  };
  for (int j = 1; j <= 18; ++j) {
    matmul(term, X, tmp);
    for (size_t i = 0; i < tmp.size(); ++i) {
      term[i] = tmp[i] / double(j);
      E[i] += term[i];
    }
  }
  for (int q = 0; q < s; ++q) {
    matmul(E, E, tmp);
    E.swap(tmp);
  }
  return E;
}

namespace {

struct Vecs {
  nsg_ctx* c;
  std::vector<nsg_tensor*> v;
  explicit Vecs(nsg_ctx* cc) : c(cc) {}
  ~Vecs() {
    for (auto* t : v) free_tensor(c, t);
  }
  nsg_tensor* add(const nsg_tensor* like) {
    v.push_back(new_tensor(c, like->dtype, like->rank, like->dims, false));
    return v.back();
  }
};

// One Lanczos expansion: given V[0..j] (orthonormal), computes w, alpha_j, beta_j.
void lanczos_step(nsg_ctx* c, nsg_linmap* m, std::vector<nsg_tensor*>& V, int j, nsg_tensor* w,
                  const std::vector<double>& beta, double* alpha_j, double* beta_j) {
  const int dt = w->dtype;
  const int64_t n = w->size;
  linmap_apply(c, m, V[j], w);
  if (j > 0) axpby(c, dt, n, -beta[j - 1], 0.0, V[j - 1]->data, 1.0, 0.0, w->data);
  std::vector<const void*> ptrs(j + 1);
  for (int i = 0; i <= j; ++i) ptrs[i] = V[i]->data;
  std::vector<double> co(2 * (j + 1)), neg(2 * (j + 1));
  double a = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    multi_dot(c, dt, n, j + 1, ptrs.data(), w->data, co.data());
    for (int i = 0; i < 2 * (j + 1); ++i) neg[i] = -co[i];
    multi_axpy(c, dt, n, j + 1, ptrs.data(), neg.data(), w->data);
    a += co[2 * j];
  }
  double b = norm2(c, dt, n, w->data);
  if (!std::isfinite(a) || !std::isfinite(b)) throw Error(NSG_ERR_NONFINITE, "Lanczos: non-finite scalar");
  *alpha_j = a;
  *beta_j = b;
}

// The Lanczos steps of one cycle with every scalar kept on the device: the two CGS
// passes' coefficients and the sum of squares of w stay in `scal` (one block of
// 4 (j + 1) + 2 doubles per step j, at step_offset(j)) and the next basis vector is
// normalised by a kernel that reads that sum of squares, so the cycle issues no host
// synchronisation; the host reads every scalar back once.  The kernels and the operand
// order are those of lanczos_step, hence the same vectors.  All K steps run; steps after
// a breakdown are discarded by the caller.
static size_t step_offset(int j) { return size_t(2) * j * (j + 1) + size_t(2) * j; }  // sum_{i<j} (4 (i+1) + 2)
void lanczos_cycle_dev(nsg_ctx* c, nsg_linmap* m, std::vector<nsg_tensor*>& V, int K, nsg_tensor* w, double* scal) {
  const int dt = w->dtype;
  const int64_t n = w->size;
  std::vector<const void*> ptrs;
  for (int j = 0; j < K; ++j) {
    double* blk = scal + step_offset(j);
    double* co1 = blk;
    double* co2 = blk + 2 * (j + 1);
    double* ss = blk + 4 * (j + 1);
    linmap_apply(c, m, V[j], w);
    if (j > 0) axpby_devscalar(c, dt, n, scal + step_offset(j - 1) + 4 * j, 1, V[j - 1]->data, w->data);
    ptrs.assign(j + 1, nullptr);
    for (int i = 0; i <= j; ++i) ptrs[i] = V[i]->data;
    multi_dot_dev(c, dt, n, j + 1, ptrs.data(), w->data, co1);
    multi_axpy_devcoef(c, dt, n, j + 1, ptrs.data(), co1, -1.0, w->data);
    multi_dot_dev(c, dt, n, j + 1, ptrs.data(), w->data, co2);
    multi_axpy_devcoef(c, dt, n, j + 1, ptrs.data(), co2, -1.0, w->data);
    const void* wp[1] = {w->data};
    multi_dot_dev(c, dt, n, 1, wp, w->data, ss);
    if (j + 1 < K) axpby_devscalar(c, dt, n, ss, 0, w->data, V[j + 1]->data);
  }
}

}  // namespace
}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_eigsolve(nsg_ctx* c, nsg_linmap* m, nsg_tensor* x, int krylovdim, int maxiter, double tol, double* eigval,
                 int* numops) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && m && x && eigval, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(krylovdim >= 1 && krylovdim <= 64 && maxiter >= 1, NSG_ERR_INVALID, "eigsolve: krylovdim 1..64");
  const int dt = x->dtype;
  const int64_t n = x->size;
  Vecs store(c);
  std::vector<nsg_tensor*> V;
  for (int i = 0; i < krylovdim; ++i) V.push_back(store.add(x));
  nsg_tensor* w = store.add(x);
  int ops = 0;
  double lam = 0.0;
  if (maxiter == 1) {
    // One cycle (the reference's default, maxiter 1): device-resident scalars and one
    // host read.  Falls through to the synchronous form below when the start vector's or
    // a kept step's sum of squares leaves the range where sqrt(sum) is exact enough
    // (the synchronous norm rescales there) -- the same arithmetic otherwise.
    const size_t nscal = step_offset(krylovdim) + 2;
    ScopedBuf sb(c, sizeof(double) * nscal);
    double* scal = (double*)sb.p;
    double* sx = scal + step_offset(krylovdim);
    const void* xp[1] = {x->data};
    multi_dot_dev(c, dt, n, 1, xp, x->data, sx);
    axpby_devscalar(c, dt, n, sx, 0, x->data, V[0]->data);
    lanczos_cycle_dev(c, m, V, krylovdim, w, scal);
    std::vector<double> hs(nscal);
    NSG_CUDA(cudaMemcpyAsync(hs.data(), scal, sizeof(double) * nscal, cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
    auto in_range = [](double q) { return std::isfinite(q) && q > 1e-280 && q < 1e280; };
    bool ok = in_range(hs[step_offset(krylovdim)]);
    std::vector<double> alpha, beta;
    int k = 0;
    for (int j = 0; j < krylovdim && ok; ++j) {
      const double* blk = hs.data() + step_offset(j);
      const double a = blk[2 * j] + blk[2 * (j + 1) + 2 * j];
      const double q = blk[4 * (j + 1)];
      if (!std::isfinite(a) || !std::isfinite(q)) {
        ok = false;
        break;
      }
      const double b = std::sqrt(q);
      alpha.push_back(a);
      beta.push_back(b);
      k = j + 1;
      if (j + 1 == krylovdim || b <= tol) break;
      if (!in_range(q)) ok = false;
    }
    if (ok) {
      ops = k;
      std::vector<double> ev(k), Y(size_t(k) * k);
      tridiag_eig(k, alpha.data(), beta.data(), ev.data(), Y.data());
      lam = ev[0];
      std::vector<double> coef(2 * k, 0.0);
      for (int j = 0; j < k; ++j) coef[2 * j] = Y[j];
      std::vector<const void*> ptrs(k);
      for (int j = 0; j < k; ++j) ptrs[j] = V[j]->data;
      NSG_CUDA(cudaMemsetAsync(x->data, 0, x->bytes, c->stream));
      multi_axpy(c, dt, n, k, ptrs.data(), coef.data(), x->data);
      const void* xq[1] = {x->data};
      multi_dot_dev(c, dt, n, 1, xq, x->data, sx);
      axpby_devscalar(c, dt, n, sx, 0, x->data, x->data);
      *eigval = lam;
      if (numops) *numops = ops;
      check_device_flag(c);
      return NSG_OK;
    }
  }
  double nx = norm2(c, dt, n, x->data);
  NSG_CHECK(nx > 0 && std::isfinite(nx), NSG_ERR_NONFINITE, "eigsolve: zero or non-finite start vector");
  axpby(c, dt, n, 1.0 / nx, 0.0, x->data, 0.0, 0.0, V[0]->data);
  for (int it = 0; it < maxiter; ++it) {
    std::vector<double> alpha, beta;
    int k = 0;
    for (int j = 0; j < krylovdim; ++j) {
      double a, b;
      beta.resize(j + 1);
      lanczos_step(c, m, V, j, w, beta, &a, &b);
      ++ops;
      alpha.push_back(a);
      beta[j] = b;
      k = j + 1;
      if (j + 1 == krylovdim || b <= tol) break;
      axpby(c, dt, n, 1.0 / b, 0.0, w->data, 0.0, 0.0, V[j + 1]->data);
    }
    std::vector<double> ev(k), Y(size_t(k) * k);
    tridiag_eig(k, alpha.data(), beta.data(), ev.data(), Y.data());
    lam = ev[0];
    std::vector<double> coef(2 * k, 0.0);
    for (int j = 0; j < k; ++j) coef[2 * j] = Y[j];
    std::vector<const void*> ptrs(k);
    for (int j = 0; j < k; ++j) ptrs[j] = V[j]->data;
    NSG_CUDA(cudaMemsetAsync(x->data, 0, x->bytes, c->stream));
    multi_axpy(c, dt, n, k, ptrs.data(), coef.data(), x->data);
    double nr = norm2(c, dt, n, x->data);
    axpby(c, dt, n, 1.0 / nr, 0.0, x->data, 0.0, 0.0, x->data);
    if (std::fabs(beta[k - 1] * Y[k - 1]) <= tol || it + 1 == maxiter) break;
    NSG_CUDA(cudaMemcpyAsync(V[0]->data, x->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  *eigval = lam;
  if (numops) *numops = ops;
  NSG_API_END(c)
}

int nsg_exponentiate(nsg_ctx* c, nsg_linmap* m, double t_re, double t_im, nsg_tensor* x, int krylovdim,
                     int maxiter, double tol, int* converged, int* numops) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && m && x, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(krylovdim >= 1 && krylovdim <= 64 && maxiter >= 1, NSG_ERR_INVALID, "exponentiate: krylovdim 1..64");
  NSG_CHECK(t_im == 0.0 || x->dtype == NSG_C128, NSG_ERR_INVALID, "exponentiate: complex time needs a complex vector");
  const int dt = x->dtype;
  const int64_t n = x->size;
  using cd = std::complex<double>;
  const cd t(t_re, t_im);
  int ops = 0;
  if (converged) *converged = 1;
  if (std::abs(t) == 0.0) {
    if (numops) *numops = 0;
    return NSG_OK;
  }
  Vecs store(c);
  std::vector<nsg_tensor*> V;
  for (int i = 0; i < krylovdim; ++i) V.push_back(store.add(x));
  nsg_tensor* w = store.add(x);
  cd remaining = t;
  bool done = false;
  for (int it = 0; it < maxiter && !done; ++it) {
    std::vector<double> alpha, beta;
    std::vector<cd> E;  // first column of exp(tau T_k)
    double err = INFINITY;
    int k = 0;
    auto expm_col = [&](int kk, cd tau, std::vector<cd>& col) {
      std::vector<cd> A(size_t(kk) * kk, cd(0, 0));
      for (int i = 0; i < kk; ++i) {
        A[i + size_t(kk) * i] = tau * alpha[i];
        if (i + 1 < kk) A[i + size_t(kk) * (i + 1)] = A[(i + 1) + size_t(kk) * i] = tau * beta[i];
      }
      std::vector<cd> E2 = expm_small(kk, A);
      col.assign(E2.begin(), E2.begin() + kk);
    };
    // Speculative device-resident cycle: the number of steps the previous cycle needed
    // (plus one) runs without host synchronisation, then the host replays the stopping
    // rule on the read-back scalars.  The vectors are those of the step-by-step form
    // (same kernels and arithmetic), so a rule that stops within the speculated steps
    // gives the identical result; a rule that has not stopped continues step by step from
    // there, and a sum of squares outside the range of an exact square root restarts the
    // cycle step by step.
    double beta0 = 0.0;
    const int spec = std::min(krylovdim, std::max(2, c->krylov_hint + 1));
    const int ops_before = ops;
    bool spec_ok = false;  // the stopping rule fired within the speculated steps
    int resume = 0;        // > 0: steps 0..resume-1 are valid, continue from step `resume`
    {
      const size_t nscal = step_offset(spec) + 2;
      ScopedBuf sb(c, sizeof(double) * nscal);
      double* scal = (double*)sb.p;
      double* sx = scal + step_offset(spec);
      const void* xp[1] = {x->data};
      multi_dot_dev(c, dt, n, 1, xp, x->data, sx);
      axpby_devscalar(c, dt, n, sx, 0, x->data, V[0]->data);
      lanczos_cycle_dev(c, m, V, spec, w, scal);
      std::vector<double> hs(nscal);
      NSG_CUDA(cudaMemcpyAsync(hs.data(), scal, sizeof(double) * nscal, cudaMemcpyDeviceToHost, c->stream));
      NSG_CUDA(cudaStreamSynchronize(c->stream));
      auto in_range = [](double q) { return std::isfinite(q) && q > 1e-280 && q < 1e280; };
      const double qx = hs[step_offset(spec)];
      if (qx == 0.0) break;
      if (in_range(qx)) {
        beta0 = std::sqrt(qx);
        for (int j = 0; j < spec; ++j) {
          const double* blk = hs.data() + step_offset(j);
          const double a = blk[2 * j] + blk[2 * (j + 1) + 2 * j];
          const double q = blk[4 * (j + 1)];
          if (!std::isfinite(a) || !std::isfinite(q)) break;
          const double b = std::sqrt(q);
          alpha.push_back(a);
          beta.push_back(b);
          ++ops;
          k = j + 1;
          expm_col(k, remaining, E);
          err = beta0 * b * std::abs(E[k - 1]);
          if (err <= tol || b <= tol * 1e-3 || j + 1 == krylovdim) {
            spec_ok = true;
            break;
          }
          if (!in_range(q)) break;
          if (j + 1 == spec) resume = spec;  // not converged yet: w holds step spec-1's vector
        }
      }
    }
    if (!spec_ok && resume > 0) {
      // continue step by step: the next basis vector from w, as the step-by-step form does
      axpby(c, dt, n, 1.0 / beta[resume - 1], 0.0, w->data, 0.0, 0.0, V[resume]->data);
    } else if (!spec_ok) {
      alpha.clear();
      beta.clear();
      ops = ops_before;
      k = 0;
      err = INFINITY;
      beta0 = norm2(c, dt, n, x->data);
      if (beta0 == 0.0) break;
      NSG_CHECK(std::isfinite(beta0), NSG_ERR_NONFINITE, "exponentiate: non-finite vector");
      axpby(c, dt, n, 1.0 / beta0, 0.0, x->data, 0.0, 0.0, V[0]->data);
    }
    for (int j = spec_ok ? krylovdim : resume; j < krylovdim; ++j) {
      double a, b;
      beta.resize(j + 1);
      lanczos_step(c, m, V, j, w, beta, &a, &b);
      ++ops;
      alpha.push_back(a);
      beta[j] = b;
      k = j + 1;
      expm_col(k, remaining, E);
      err = beta0 * b * std::abs(E[k - 1]);
      if (err <= tol || b <= tol * 1e-3 || j + 1 == krylovdim) break;
      axpby(c, dt, n, 1.0 / b, 0.0, w->data, 0.0, 0.0, V[j + 1]->data);
    }
    c->krylov_hint = k;
    cd step = remaining;
    if (!(err <= tol || beta[k - 1] <= tol * 1e-3)) {
      // largest fraction of the remaining step within the per-unit-time error budget
      auto est = [&](double s, std::vector<cd>& col) {
        expm_col(k, remaining * s, col);
        return beta0 * beta[k - 1] * std::abs(col[k - 1]);
      };
      double lo = 0.0, hi = 1.0;
      std::vector<cd> tmp;
      for (int b = 0; b < 50; ++b) {
        double mid = 0.5 * (lo + hi);
        if (est(mid, tmp) <= tol * mid * std::abs(remaining) / std::abs(t))
          lo = mid;
        else
          hi = mid;
      }
      if (lo <= 0.0) break;
      step = remaining * lo;
      est(lo, E);
    }
    std::vector<double> coef(2 * k);
    for (int j = 0; j < k; ++j) {
      cd cj = beta0 * E[j];
      coef[2 * j] = cj.real();
      coef[2 * j + 1] = cj.imag();
    }
    std::vector<const void*> ptrs(k);
    for (int j = 0; j < k; ++j) ptrs[j] = V[j]->data;
    NSG_CUDA(cudaMemsetAsync(x->data, 0, x->bytes, c->stream));
    multi_axpy(c, dt, n, k, ptrs.data(), coef.data(), x->data);
    remaining -= step;
    if (std::abs(remaining) <= 1e-15 * std::abs(t)) done = true;
  }
  if (converged) *converged = done ? 1 : 0;
  if (numops) *numops = ops;
  NSG_API_END(c)
}

int nsg_runge_kutta(nsg_ctx* c, nsg_linmap* m, double t_re, double t_im, nsg_tensor* x, int order) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && m && x, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(order == 2 || order == 4, NSG_ERR_INVALID, "For runge_kutta_solver, must specify `order` keyword");
  NSG_CHECK(t_im == 0.0 || x->dtype == NSG_C128, NSG_ERR_INVALID, "runge_kutta: complex time needs a complex vector");
  const int dt = x->dtype;
  const int64_t n = x->size;
  Vecs store(c);
  nsg_tensor* k1 = store.add(x);
  nsg_tensor* kb = store.add(x);
  nsg_tensor* tmp = store.add(x);
  std::complex<double> t(t_re, t_im);
  if (order == 2) {
    linmap_apply(c, m, x, k1);    // H psi
    linmap_apply(c, m, k1, tmp);  // H^2 psi
    std::complex<double> h2 = t * t / 2.0;
    axpby(c, dt, n, t.real(), t.imag(), k1->data, 1.0, 0.0, x->data);
    axpby(c, dt, n, h2.real(), h2.imag(), tmp->data, 1.0, 0.0, x->data);
    return NSG_OK;
  }
  nsg_tensor* acc = store.add(x);
  std::complex<double> h = t / 2.0, t6 = t / 6.0;
  linmap_apply(c, m, x, k1);  // k1 = H psi
  NSG_CUDA(cudaMemcpyAsync(acc->data, k1->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  // k2 = k1 + (t/2) H k1
  linmap_apply(c, m, k1, tmp);
  NSG_CUDA(cudaMemcpyAsync(kb->data, k1->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  axpby(c, dt, n, h.real(), h.imag(), tmp->data, 1.0, 0.0, kb->data);
  axpby(c, dt, n, 2.0, 0.0, kb->data, 1.0, 0.0, acc->data);
  // k3 = k1 + (t/2) H k2
  linmap_apply(c, m, kb, tmp);
  NSG_CUDA(cudaMemcpyAsync(kb->data, k1->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  axpby(c, dt, n, h.real(), h.imag(), tmp->data, 1.0, 0.0, kb->data);
  axpby(c, dt, n, 2.0, 0.0, kb->data, 1.0, 0.0, acc->data);
  // k4 = k1 + t H k3
  linmap_apply(c, m, kb, tmp);
  NSG_CUDA(cudaMemcpyAsync(kb->data, k1->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  axpby(c, dt, n, t.real(), t.imag(), tmp->data, 1.0, 0.0, kb->data);
  axpby(c, dt, n, 1.0, 0.0, kb->data, 1.0, 0.0, acc->data);
  // psi += (t/6) acc
  axpby(c, dt, n, t6.real(), t6.imag(), acc->data, 1.0, 0.0, x->data);
  NSG_API_END(c)
}

}  // extern "C"
