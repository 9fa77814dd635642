// Memory-bound kernels: permutation, axpby, batched dot products (Lanczos
// reorthogonalisation), fused multi-axpy, norms, gathers and concatenation.
//
// All reductions are two-stage with a fixed summation order, so results are
// bit-reproducible run to run (no floating-point atomics).
#include "nsg_internal.h"

#include <cmath>

namespace nsg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double conjv(double v) { return v; }
__device__ __forceinline__ double2 conjv(double2 v) { return make_double2(v.x, -v.y); }

inline int grid_for(nsg_ctx* c, int64_t n, int per_sm = 8) {
  int64_t blocks = (n + kThreads - 1) / kThreads;
  int64_t cap = int64_t(c->num_sms > 0 ? c->num_sms : 152) * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return int(blocks);
}

// ---------------------------------------------------------------------------
struct PermParams {
  int rank;
  int64_t odims[NSG_MAX_RANK];
  int64_t istride[NSG_MAX_RANK];  // input stride of the input axis feeding output axis k
};

template <typename T, bool CONJ>
__global__ void __launch_bounds__(kThreads)
    permute_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n, PermParams p) {
  for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < n; o += int64_t(gridDim.x) * blockDim.x) {
    int64_t rem = o, src = 0;
    for (int k = 0; k < p.rank; ++k) {
      int64_t d = p.odims[k];
      int64_t i = rem % d;
      rem /= d;
      src += i * p.istride[k];
    }
    T v = in[src];
    if constexpr (CONJ) v = conjv(v);
    out[o] = v;
  }
}

// Tiled transpose for in[a + A*(b + B*c)] -> out[b + B*(a + A*c)] (32x32 tiles), the
// case where the fastest output axis group is not the fastest input group.
template <typename T, bool CONJ>
__global__ void __launch_bounds__(kThreads)
    transpose3_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t A, int64_t B, int64_t Cn) {
  __shared__ T tile[32][33];
  int64_t ntA = (A + 31) / 32, ntB = (B + 31) / 32;
  int64_t ntiles = ntA * ntB * Cn;
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int64_t ta = t % ntA, tb = (t / ntA) % ntB, cc = t / (ntA * ntB);
    for (int r = ty; r < 32; r += 8) {
      int64_t a = ta * 32 + tx, b = tb * 32 + r;
      if (a < A && b < B) tile[r][tx] = in[a + A * (b + B * cc)];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      int64_t b = tb * 32 + tx, a = ta * 32 + r;
      if (a < A && b < B) {
        T v = tile[tx][r];
        if constexpr (CONJ) v = conjv(v);
        out[b + B * (a + A * cc)] = v;
      }
    }
    __syncthreads();
  }
}

__global__ void axpby_real_kernel(int64_t n, double a, const double* __restrict__ x, double b,
                                  double* __restrict__ y) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = (b == 0.0 ? a * x[i] : fma(a, x[i], b * y[i]));
}

__global__ void axpby_cplx_kernel(int64_t n, double2 a, const double2* __restrict__ x, double2 b,
                                  double2* __restrict__ y) {
  bool bz = (b.x == 0.0 && b.y == 0.0);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double2 ax = cmul(a, x[i]);
    if (!bz) {
      double2 by = cmul(b, y[i]);
      ax.x += by.x;
      ax.y += by.y;
    }
    y[i] = ax;
  }
}

struct VecPtrs {
  const void* v[64];
};

// partial dot products <v_j, w>: blockIdx.y = j; partial[(j * gridDim.x + blockIdx.x)] (re, im)
template <bool CPLX>
__global__ void __launch_bounds__(kThreads)
    dot_partial_kernel(int64_t n, VecPtrs vp, const void* w_, double* partial) {
  __shared__ double sre[kThreads], sim[kThreads];
  int j = blockIdx.y;
  double re = 0.0, im = 0.0;
  if constexpr (CPLX) {
    const double2* v = (const double2*)vp.v[j];
    const double2* w = (const double2*)w_;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
      double2 a = v[i], b = w[i];
      re = fma(a.x, b.x, fma(a.y, b.y, re));
      im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
  } else {
    const double* v = (const double*)vp.v[j];
    const double* w = (const double*)w_;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
      re = fma(v[i], w[i], re);
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sre[threadIdx.x] += sre[threadIdx.x + s];
      sim[threadIdx.x] += sim[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    size_t o = 2 * (size_t(j) * gridDim.x + blockIdx.x);
    partial[o] = sre[0];
    partial[o + 1] = sim[0];
  }
}

// one warp per vector; fixed order
__global__ void dot_final_kernel(int nb, const double* partial, double* out) {
  int j = blockIdx.x;
  int lane = threadIdx.x;
  double re = 0.0, im = 0.0;
  for (int b = lane; b < nb; b += 32) {
    re += partial[2 * (size_t(j) * nb + b)];
    im += partial[2 * (size_t(j) * nb + b) + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  if (lane == 0) {
    out[2 * j] = re;
    out[2 * j + 1] = im;
  }
}

struct AxpyParams {
  const void* v[64];
  double coef[128];
};

template <bool CPLX>
__global__ void __launch_bounds__(kThreads) multi_axpy_kernel(int64_t n, int nv, AxpyParams p, void* w_) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    if constexpr (CPLX) {
      double2* w = (double2*)w_;
      double2 acc = w[i];
      for (int j = 0; j < nv; ++j) {
        double2 a = ((const double2*)p.v[j])[i];
        double cr = p.coef[2 * j], ci = p.coef[2 * j + 1];
        acc.x = fma(cr, a.x, fma(-ci, a.y, acc.x));
        acc.y = fma(cr, a.y, fma(ci, a.x, acc.y));
      }
      w[i] = acc;
    } else {
      double* w = (double*)w_;
      double acc = w[i];
      for (int j = 0; j < nv; ++j) acc = fma(p.coef[2 * j], ((const double*)p.v[j])[i], acc);
      w[i] = acc;
    }
  }
}

// multi_axpy with coefficients read from device memory, scaled by `sign` (+1 or -1:
// exact), in the arithmetic of multi_axpy_kernel
template <bool CPLX>
__global__ void __launch_bounds__(kThreads)
    multi_axpy_devcoef_kernel(int64_t n, int nv, VecPtrs vp, const double* __restrict__ coef, double sign, void* w_) {
  __shared__ double cs[128];
  for (int j = threadIdx.x; j < 2 * nv; j += blockDim.x) cs[j] = sign * coef[j];
  __syncthreads();
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    if constexpr (CPLX) {
      double2* w = (double2*)w_;
      double2 acc = w[i];
      for (int j = 0; j < nv; ++j) {
        double2 a = ((const double2*)vp.v[j])[i];
        double cr = cs[2 * j], ci = cs[2 * j + 1];
        acc.x = fma(cr, a.x, fma(-ci, a.y, acc.x));
        acc.y = fma(cr, a.y, fma(ci, a.x, acc.y));
      }
      w[i] = acc;
    } else {
      double* w = (double*)w_;
      double acc = w[i];
      for (int j = 0; j < nv; ++j) acc = fma(cs[2 * j], ((const double*)vp.v[j])[i], acc);
      w[i] = acc;
    }
  }
}

// y = a x + b y with a, b from a device sum of squares s (in the arithmetic of the
// axpby kernels): mode 0: a = 1 / sqrt(s), b = 0 (normalise); mode 1: a = -sqrt(s), b = 1
template <bool CPLX>
__global__ void axpby_devscalar_kernel(int64_t n, const double* __restrict__ s_dev, int mode, const void* x_, void* y_) {
  const double nr = sqrt(s_dev[0]);
  const double a = mode == 0 ? 1.0 / nr : -nr;
  const double b = mode == 0 ? 0.0 : 1.0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    if constexpr (CPLX) {
      const double2* x = (const double2*)x_;
      double2* y = (double2*)y_;
      double2 ax = cmul(make_double2(a, 0.0), x[i]);
      if (b != 0.0) {
        double2 by = cmul(make_double2(b, 0.0), y[i]);
        ax.x += by.x;
        ax.y += by.y;
      }
      y[i] = ax;
    } else {
      const double* x = (const double*)x_;
      double* y = (double*)y_;
      y[i] = (b == 0.0 ? a * x[i] : fma(a, x[i], b * y[i]));
    }
  }
}

template <typename T>
__global__ void copy_columns_kernel(int64_t rows, int64_t ncols, const T* __restrict__ src, int64_t lds,
                                    const int* __restrict__ colidx, T* __restrict__ dst, int64_t ldd) {
  int64_t n = rows * ncols;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = e % rows, k = e / rows;
    int64_t sc = colidx ? colidx[k] : k;
    dst[i + k * ldd] = src[i + sc * lds];
  }
}

template <bool CPLX>
__global__ void row_norms_kernel(int64_t rows, int64_t cols, const void* A_, int64_t lda, double* out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < rows; i += int64_t(gridDim.x) * blockDim.x) {
    double s = 0.0;
    if constexpr (CPLX) {
      const double2* A = (const double2*)A_;
      for (int64_t j = 0; j < cols; ++j) {
        double2 a = A[i + j * lda];
        s = fma(a.x, a.x, fma(a.y, a.y, s));
      }
    } else {
      const double* A = (const double*)A_;
      for (int64_t j = 0; j < cols; ++j) {
        double a = A[i + j * lda];
        s = fma(a, a, s);
      }
    }
    out[i] = s;
  }
}

__global__ void amax_partial_kernel(int64_t n, const double* __restrict__ x, double* __restrict__ partial) {
  __shared__ double red[kThreads];
  double m = 0.0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    m = fmax(m, fabs(x[i]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

template <typename T>
__global__ void concat_kernel(int64_t pre, int64_t Ka, int64_t Kb, int64_t post, const T* __restrict__ a,
                              const T* __restrict__ b, T* __restrict__ out) {
  int64_t K = Ka + Kb, n = pre * K * post;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t p = e % pre, k = (e / pre) % K, q = e / (pre * K);
    out[e] = k < Ka ? a[p + pre * (k + Ka * q)] : b[p + pre * ((k - Ka) + Kb * q)];
  }
}

template <typename T, bool CONJ>
void launch_permute(nsg_ctx* c, const nsg_tensor* x, nsg_tensor* out, const int* perm) {
  int r = x->rank;
  int64_t instr[NSG_MAX_RANK];
  int64_t s = 1;
  for (int k = 0; k < r; ++k) {
    instr[k] = s;
    s *= x->dims[k];
  }
  // perm = [j, j+1, ..., k-1, 0, ..., j-1, k, ..., r-1]  ->  3-block tiled transpose
  int j = perm[0];
  if (j > 0) {
    int L = 1;
    while (L < r && perm[L] == j + L) ++L;
    int k = j + L;
    bool ok = (L + j <= r);
    for (int t = 0; ok && t < j; ++t) ok = (perm[L + t] == t);
    for (int t = L + j; ok && t < r; ++t) ok = (perm[t] == t);
    if (ok) {
      int64_t A = 1, B = 1, Cn = 1;
      for (int t = 0; t < j; ++t) A *= x->dims[t];
      for (int t = j; t < k; ++t) B *= x->dims[t];
      for (int t = k; t < r; ++t) Cn *= x->dims[t];
      int64_t tiles = ((A + 31) / 32) * ((B + 31) / 32) * Cn;
      int64_t cap = int64_t(c->num_sms) * 16;
      int grid = int(tiles < cap ? tiles : cap);
      if (grid < 1) grid = 1;
      transpose3_kernel<T, CONJ><<<grid, kThreads, 0, c->stream>>>((const T*)x->data, (T*)out->data, A, B, Cn);
      count_launch(c);
      check_launch("transpose3");
      return;
    }
  }
  PermParams p;
  p.rank = r;
  for (int k = 0; k < r; ++k) {
    p.odims[k] = x->dims[perm[k]];
    p.istride[k] = instr[perm[k]];
  }
  permute_kernel<T, CONJ><<<grid_for(c, x->size), kThreads, 0, c->stream>>>((const T*)x->data, (T*)out->data,
                                                                          x->size, p);
  count_launch(c);
  check_launch("permute");
}

}  // namespace

// ---------------------------------------------------------------------------

void permute(nsg_ctx* c, const nsg_tensor* x, const int* perm, bool conj, nsg_tensor* out) {
  bool ident = true;
  for (int k = 0; k < x->rank; ++k) ident &= (perm[k] == k);
  bool cplx = x->dtype == NSG_C128;
  if (ident && !(conj && cplx)) {
    NSG_CUDA(cudaMemcpyAsync(out->data, x->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
    return;
  }
  if (cplx) {
    if (conj)
      launch_permute<double2, true>(c, x, out, perm);
    else
      launch_permute<double2, false>(c, x, out, perm);
  } else {
    launch_permute<double, false>(c, x, out, perm);
  }
}

void axpby(nsg_ctx* c, int dtype, int64_t n, double ar, double ai, const void* x, double br, double bi,
           void* y) {
  int grid = grid_for(c, n);
  if (dtype == NSG_C128)
    axpby_cplx_kernel<<<grid, kThreads, 0, c->stream>>>(n, make_double2(ar, ai), (const double2*)x,
                                                        make_double2(br, bi), (double2*)y);
  else
    axpby_real_kernel<<<grid, kThreads, 0, c->stream>>>(n, ar, (const double*)x, br, (double*)y);
  count_launch(c);
  check_launch("axpby");
}

void scale(nsg_ctx* c, int dtype, int64_t n, double ar, double ai, void* x) {
  axpby(c, dtype, n, ar, ai, x, 0.0, 0.0, x);
}

void multi_dot(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const void* w, double* host_out) {
  NSG_CHECK(nv >= 1 && nv <= 64, NSG_ERR_INVALID, "multi_dot: 1..64 vectors");
  int nb = grid_for(c, n, 2);
  if (nb > 256) nb = 256;
  double* scratch = dev_scratch(c, size_t(2) * nb * nv + 2 * nv);
  double* out_dev = scratch + size_t(2) * nb * nv;
  VecPtrs vp;
  for (int j = 0; j < nv; ++j) vp.v[j] = v[j];
  dim3 grid(nb, nv);
  if (dtype == NSG_C128)
    dot_partial_kernel<true><<<grid, kThreads, 0, c->stream>>>(n, vp, w, scratch);
  else
    dot_partial_kernel<false><<<grid, kThreads, 0, c->stream>>>(n, vp, w, scratch);
  dot_final_kernel<<<nv, 32, 0, c->stream>>>(nb, scratch, out_dev);
  count_launch(c, 2);
  check_launch("multi_dot");
  double* h = host_scalars(c, 2 * nv);
  NSG_CUDA(cudaMemcpyAsync(h, out_dev, sizeof(double) * 2 * nv, cudaMemcpyDeviceToHost, c->stream));
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  for (int j = 0; j < 2 * nv; ++j) host_out[j] = h[j];
}

void multi_axpy(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const double* coef, void* w) {
  NSG_CHECK(nv >= 0 && nv <= 64, NSG_ERR_INVALID, "multi_axpy: 0..64 vectors");
  if (nv == 0) return;
  AxpyParams p;
  for (int j = 0; j < nv; ++j) {
    p.v[j] = v[j];
    p.coef[2 * j] = coef[2 * j];
    p.coef[2 * j + 1] = coef[2 * j + 1];
  }
  int grid = grid_for(c, n);
  if (dtype == NSG_C128)
    multi_axpy_kernel<true><<<grid, kThreads, 0, c->stream>>>(n, nv, p, w);
  else
    multi_axpy_kernel<false><<<grid, kThreads, 0, c->stream>>>(n, nv, p, w);
  count_launch(c);
  check_launch("multi_axpy");
}

void multi_dot_dev(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const void* w, double* out_dev) {
  NSG_CHECK(nv >= 1 && nv <= 64, NSG_ERR_INVALID, "multi_dot: 1..64 vectors");
  int nb = grid_for(c, n, 2);
  if (nb > 256) nb = 256;
  double* scratch = dev_scratch(c, size_t(2) * nb * nv);
  VecPtrs vp;
  for (int j = 0; j < nv; ++j) vp.v[j] = v[j];
  dim3 grid(nb, nv);
  if (dtype == NSG_C128)
    dot_partial_kernel<true><<<grid, kThreads, 0, c->stream>>>(n, vp, w, scratch);
  else
    dot_partial_kernel<false><<<grid, kThreads, 0, c->stream>>>(n, vp, w, scratch);
  dot_final_kernel<<<nv, 32, 0, c->stream>>>(nb, scratch, out_dev);
  count_launch(c, 2);
  check_launch("multi_dot_dev");
}

void multi_axpy_devcoef(nsg_ctx* c, int dtype, int64_t n, int nv, const void* const* v, const double* coef_dev,
                        double sign, void* w) {
  NSG_CHECK(nv >= 1 && nv <= 64, NSG_ERR_INVALID, "multi_axpy: 1..64 vectors");
  VecPtrs vp;
  for (int j = 0; j < nv; ++j) vp.v[j] = v[j];
  int grid = grid_for(c, n);
  if (dtype == NSG_C128)
    multi_axpy_devcoef_kernel<true><<<grid, kThreads, 0, c->stream>>>(n, nv, vp, coef_dev, sign, w);
  else
    multi_axpy_devcoef_kernel<false><<<grid, kThreads, 0, c->stream>>>(n, nv, vp, coef_dev, sign, w);
  count_launch(c);
  check_launch("multi_axpy_devcoef");
}

void axpby_devscalar(nsg_ctx* c, int dtype, int64_t n, const double* s_dev, int mode, const void* x, void* y) {
  int grid = grid_for(c, n);
  if (dtype == NSG_C128)
    axpby_devscalar_kernel<true><<<grid, kThreads, 0, c->stream>>>(n, s_dev, mode, x, y);
  else
    axpby_devscalar_kernel<false><<<grid, kThreads, 0, c->stream>>>(n, s_dev, mode, x, y);
  count_launch(c);
  check_launch("axpby_devscalar");
}

double norm2(nsg_ctx* c, int dtype, int64_t n, const void* x) {
  double out[2];
  const void* v[1] = {x};
  multi_dot(c, dtype, n, 1, v, x, out);
  if (std::isfinite(out[0]) && out[0] > 1e-280) return std::sqrt(out[0]);
  // overflow or underflow of the sum of squares: rescale by the largest component
  double mx = amax(c, dtype, n, x);
  if (mx == 0.0 || !std::isfinite(mx)) return mx;
  int64_t nd = dtype == NSG_C128 ? 2 * n : n;
  double* tmp = (double*)dalloc(c, sizeof(double) * nd);
  axpby(c, NSG_F64, nd, 1.0 / mx, 0.0, x, 0.0, 0.0, tmp);
  const void* vt[1] = {tmp};
  multi_dot(c, NSG_F64, nd, 1, vt, tmp, out);
  dfree(c, tmp, sizeof(double) * nd);
  return mx * std::sqrt(out[0] > 0 ? out[0] : 0.0);
}

void copy_columns(nsg_ctx* c, int dtype, int64_t rows, int64_t ncols, const void* src, int64_t lds,
                  const int* d_colidx, void* dst, int64_t ldd) {
  if (rows * ncols == 0) return;
  int grid = grid_for(c, rows * ncols);
  if (dtype == NSG_C128)
    copy_columns_kernel<double2><<<grid, kThreads, 0, c->stream>>>(rows, ncols, (const double2*)src, lds, d_colidx,
                                                                  (double2*)dst, ldd);
  else
    copy_columns_kernel<double><<<grid, kThreads, 0, c->stream>>>(rows, ncols, (const double*)src, lds, d_colidx,
                                                                 (double*)dst, ldd);
  count_launch(c);
  check_launch("copy_columns");
}

void copy_rows(nsg_ctx* c, int dtype, int64_t nrows_out, int64_t ncols, const void* src, int64_t lds, void* dst,
               int64_t ldd) {
  // rows [0, nrows_out) of a column-major matrix = a strided 2-D copy
  size_t eb = elem_bytes(dtype);
  NSG_CUDA(cudaMemcpy2DAsync(dst, ldd * eb, src, lds * eb, nrows_out * eb, ncols, cudaMemcpyDeviceToDevice,
                             c->stream));
}

double amax(nsg_ctx* c, int dtype, int64_t n, const void* x) {
  // complex: max over real and imaginary parts (a factor sqrt(2) of the modulus at most)
  int64_t nd = dtype == NSG_C128 ? 2 * n : n;
  int nb = grid_for(c, nd, 2);
  double* scratch = dev_scratch(c, nb);
  amax_partial_kernel<<<nb, kThreads, 0, c->stream>>>(nd, (const double*)x, scratch);
  count_launch(c);
  check_launch("amax");
  std::vector<double> h(nb);
  NSG_CUDA(cudaMemcpyAsync(h.data(), scratch, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  double m = 0.0;
  for (double v : h) m = std::fmax(m, v);
  return m;
}

void row_norms2(nsg_ctx* c, int dtype, int64_t rows, int64_t cols, const void* A, int64_t lda, double* out_dev) {
  int grid = grid_for(c, rows);
  if (dtype == NSG_C128)
    row_norms_kernel<true><<<grid, kThreads, 0, c->stream>>>(rows, cols, A, lda, out_dev);
  else
    row_norms_kernel<false><<<grid, kThreads, 0, c->stream>>>(rows, cols, A, lda, out_dev);
  count_launch(c);
  check_launch("row_norms");
}

}  // namespace nsg

using namespace nsg;

// dst(r0d + i, c0d + j) (+)= src(r0s + i, c0s + j) for i < rows, j < cols, both tensors
// viewed as column-major matrices with the given leading dimensions
template <typename T, bool ACC>
__global__ void copy_submatrix_kernel(const T* __restrict__ src, int64_t lds, T* __restrict__ dst, int64_t ldd,
                                      int64_t rows, int64_t cols) {
  const int64_t tot = rows * cols;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = e % rows, j = e / rows;
    const T v = src[i + j * lds];
    if constexpr (ACC) {
      if constexpr (sizeof(T) == 8) {
        dst[i + j * ldd] += v;
      } else {
        T& d = dst[i + j * ldd];
        d.x += v.x;
        d.y += v.y;
      }
    } else {
      dst[i + j * ldd] = v;
    }
  }
}

extern "C" int nsg_copy_submatrix(nsg_ctx* c, const nsg_tensor* src, int64_t lds, int64_t r0s, int64_t c0s,
                                  nsg_tensor* dst, int64_t ldd, int64_t r0d, int64_t c0d, int64_t rows, int64_t cols,
                                  int accumulate) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && src && dst, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(src->dtype == dst->dtype, NSG_ERR_INVALID, "copy_submatrix: dtypes differ");
  NSG_CHECK(rows >= 0 && cols >= 0 && lds >= 1 && ldd >= 1 && r0s >= 0 && c0s >= 0 && r0d >= 0 && c0d >= 0,
            NSG_ERR_INVALID, "copy_submatrix: negative extent or offset");
  if (rows == 0 || cols == 0) return NSG_OK;
  NSG_CHECK(r0s + rows <= lds && r0d + rows <= ldd, NSG_ERR_INVALID, "copy_submatrix: rows beyond the leading dimension");
  NSG_CHECK(r0s + rows + (c0s + cols - 1) * lds <= src->size, NSG_ERR_INVALID, "copy_submatrix: box beyond the source");
  NSG_CHECK(r0d + rows + (c0d + cols - 1) * ldd <= dst->size, NSG_ERR_INVALID,
            "copy_submatrix: box beyond the destination");
  const int grid = grid_for(c, rows * cols);
  const size_t eb = elem_bytes(src->dtype);
  const char* s = (const char*)src->data + eb * size_t(r0s + c0s * lds);
  char* d = (char*)dst->data + eb * size_t(r0d + c0d * ldd);
  if (src->dtype == NSG_C128) {
    if (accumulate)
      copy_submatrix_kernel<double2, true><<<grid, kThreads, 0, c->stream>>>((const double2*)s, lds, (double2*)d, ldd,
                                                                           rows, cols);
    else
      copy_submatrix_kernel<double2, false><<<grid, kThreads, 0, c->stream>>>((const double2*)s, lds, (double2*)d,
                                                                            ldd, rows, cols);
  } else {
    if (accumulate)
      copy_submatrix_kernel<double, true><<<grid, kThreads, 0, c->stream>>>((const double*)s, lds, (double*)d, ldd,
                                                                          rows, cols);
    else
      copy_submatrix_kernel<double, false><<<grid, kThreads, 0, c->stream>>>((const double*)s, lds, (double*)d, ldd,
                                                                           rows, cols);
  }
  count_launch(c);
  check_launch("copy_submatrix");
  NSG_API_END(c)
}

extern "C" int nsg_concat(nsg_ctx* c, const nsg_tensor* a, const nsg_tensor* b, int axis, nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && a && b && out, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(a->dtype == b->dtype && a->rank == b->rank && axis >= 0 && axis < a->rank, NSG_ERR_INVALID,
            "concat: rank/dtype/axis mismatch");
  int64_t dims[NSG_MAX_RANK];
  int64_t pre = 1, post = 1;
  for (int k = 0; k < a->rank; ++k) {
    if (k != axis) NSG_CHECK(a->dims[k] == b->dims[k], NSG_ERR_INVALID, "concat: dims differ off the axis");
    dims[k] = a->dims[k];
    if (k < axis) pre *= a->dims[k];
    if (k > axis) post *= a->dims[k];
  }
  dims[axis] = a->dims[axis] + b->dims[axis];
  nsg_tensor* t = new_tensor(c, a->dtype, a->rank, dims, false);
  int grid = grid_for(c, t->size);
  if (a->dtype == NSG_C128)
    concat_kernel<double2><<<grid, kThreads, 0, c->stream>>>(pre, a->dims[axis], b->dims[axis], post,
                                                             (const double2*)a->data, (const double2*)b->data,
                                                             (double2*)t->data);
  else
    concat_kernel<double><<<grid, kThreads, 0, c->stream>>>(pre, a->dims[axis], b->dims[axis], post,
                                                            (const double*)a->data, (const double*)b->data,
                                                            (double*)t->data);
  count_launch(c);
  check_launch("concat");
  *out = t;
  NSG_API_END(c)
}
