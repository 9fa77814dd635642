// FP64 / complex-FP64 strided-batched GEMM on the CUDA cores (the plain form).
//
// C_b = alpha * op(A_b) * op(B_b) + beta * C_b, column-major, op in {N, T, C, R}.
// GB300 executes FP64 at a small fraction of its FP32 rate, so this kernel is
// compute-bound for every shape that matters; a 64x64 tile with 4x4 outputs per
// thread keeps the FP64 pipes busy.  Loads are mapped so that consecutive threads
// touch consecutive addresses for either operand orientation.
#include "nsg_internal.h"
#include "tuning_table.h"

#include <algorithm>
#include <map>
#include <mutex>

namespace nsg {

namespace {

constexpr int BM = 64, BN = 64, NT = 256;

__device__ __forceinline__ double ld(const double* p, bool) { return *p; }
__device__ __forceinline__ double2 ld(const double2* p, bool conj) {
  double2 v = *p;
  if (conj) v.y = -v.y;
  return v;
}
__device__ __forceinline__ void zero(double& v) { v = 0.0; }
__device__ __forceinline__ bool nonzero(double v) { return v != 0.0; }
__device__ __forceinline__ bool nonzero(double2 v) { return v.x != 0.0 || v.y != 0.0; }
__device__ __forceinline__ void zero(double2& v) { v = make_double2(0.0, 0.0); }
__device__ __forceinline__ void mac(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void mac(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}

template <typename T>
struct Scal;
template <>
struct Scal<double> {
  double a, b;
  __device__ double epi(double acc, const double* c) const { return b == 0.0 ? a * acc : fma(a, acc, b * (*c)); }
};
template <>
struct Scal<double2> {
  double2 a, b;
  __device__ double2 epi(double2 acc, const double2* c) const {
    double2 r = make_double2(a.x * acc.x - a.y * acc.y, a.x * acc.y + a.y * acc.x);
    if (b.x != 0.0 || b.y != 0.0) {
      double2 cv = *c;
      r.x += b.x * cv.x - b.y * cv.y;
      r.y += b.x * cv.y + b.y * cv.x;
    }
    return r;
  }
};

// splits > 1: grid z covers batch * splits; split sp sums k in [sp*ksplit, (sp+1)*ksplit)
// and writes its raw partial product to C + bz * M * N (ld = M); a reduction applies
// alpha / beta afterwards in a fixed order.
template <typename T, int BK>
__global__ void __launch_bounds__(NT)
    gemm_kernel(int64_t M, int64_t N, int64_t Kfull, const T* __restrict__ A, int64_t lda, int64_t sA, int opA,
                const T* __restrict__ B, int64_t ldb, int64_t sB, int opB, T* __restrict__ C, int64_t ldc,
                int64_t sC, int64_t batch, Scal<T> sc, int splits, int64_t ksplit) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = int64_t(blockIdx.x) * BM, n0 = int64_t(blockIdx.y) * BN;
  const bool transA = (opA == OP_T || opA == OP_C), conjA = (opA == OP_C || opA == OP_R);
  const bool transB = (opB == OP_T || opB == OP_C), conjB = (opB == OP_C || opB == OP_R);
  for (int64_t bzz = blockIdx.z; bzz < batch * splits; bzz += gridDim.z) {
    const int64_t bz = bzz / splits, sp = bzz % splits;
    const int64_t kb = sp * ksplit;
    const int64_t K = (splits > 1) ? ((kb + ksplit < Kfull) ? ksplit : Kfull - kb) : Kfull;
    const T* Ab = A + bz * sA + (transA ? kb : kb * lda);
    const T* Bb = B + bz * sB + (transB ? kb * ldb : kb);
    T* Cb = (splits > 1) ? C + bzz * M * N : C + bz * sC;
    const int64_t ldcc = (splits > 1) ? M : ldc;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) zero(acc[i][j]);
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
      // A tile: BM x BK
#pragma unroll
      for (int r = 0; r < (BM * BK) / NT; ++r) {
        int e = threadIdx.x + r * NT;
        int i, k;
        if (!transA) {
          i = e % BM;
          k = e / BM;
        } else {
          k = e % BK;
          i = e / BK;
        }
        int64_t gi = m0 + i, gk = k0 + k;
        T v;
        zero(v);
        if (gi < M && gk < K) v = ld(transA ? Ab + gk + gi * lda : Ab + gi + gk * lda, conjA);
        As[k][i] = v;
      }
      // B tile: BK x BN
#pragma unroll
      for (int r = 0; r < (BN * BK) / NT; ++r) {
        int e = threadIdx.x + r * NT;
        int j, k;
        if (!transB) {
          k = e % BK;
          j = e / BK;
        } else {
          j = e % BN;
          k = e / BN;
        }
        int64_t gj = n0 + j, gk = k0 + k;
        T v;
        zero(v);
        if (gj < N && gk < K) v = ld(transB ? Bb + gj + gk * ldb : Bb + gk + gj * ldb, conjB);
        Bs[k][j] = v;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) mac(acc[i][j], a[i], b[j]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int64_t gi = m0 + ty + 16 * i;
      if (gi >= M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int64_t gj = n0 + tx + 16 * j;
        if (gj >= N) continue;
        T* cp = Cb + gi + gj * ldcc;
        if (splits > 1)
          *cp = acc[i][j];
        else
          *cp = sc.epi(acc[i][j], cp);
      }
    }
  }
}

template <typename T>
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int64_t batch, int splits, const T* __restrict__ W,
                                     T* __restrict__ C, int64_t ldc, int64_t sC, Scal<T> sc) {
  const int64_t MN = M * N, tot = MN * batch;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot; e += int64_t(gridDim.x) * blockDim.x) {
    int64_t b = e / MN, r = e % MN, i = r % M, j = r / M;
    T acc;
    zero(acc);
    for (int sp = 0; sp < splits; ++sp) {
      T v = W[(b * splits + sp) * MN + r];
      if constexpr (sizeof(T) == 8) {
        acc += v;
      } else {
        acc.x += v.x;
        acc.y += v.y;
      }
    }
    T* cp = C + b * sC + i + j * ldc;
    *cp = sc.epi(acc, cp);
  }
}

// Tall-skinny products with N, K <= 32: the site-operator steps of H_eff and of the
// environment updates (K, N = w d, batched over the other bond).  op(B) is an MPO
// tensor and mostly zeros, so each CTA lists its non-zeros per column (warp ballots)
// and stages a 256-row tile of op(A) in shared memory ([k][row], conflict-free); thread
// r then forms row r of C from exactly nnz(B) multiply-adds.  The FP64 work drops by
// the operator's sparsity and the kernel runs at the HBM rate of reading A and writing C.
constexpr int kSkinnyRows = 256;
template <typename T>
__global__ void __launch_bounds__(kSkinnyRows)
    gemm_skinny_kernel(int64_t M, int N, int K, const T* __restrict__ A, int64_t lda, int64_t sA, bool conjA,
                       const T* __restrict__ B, int64_t ldb, int64_t sB, int opB, T* __restrict__ C,
                       int64_t ldc, int64_t sC, int64_t batch, Scal<T> sc) {
  extern __shared__ __align__(16) unsigned char sk_smem[];
  T* As = (T*)sk_smem;                        // [K][kSkinnyRows]
  __shared__ T nzv[32 * 32];                  // non-zeros of op(B), column-major order
  __shared__ unsigned char nzk[32 * 32];      // their row index k
  __shared__ int colptr[33];
  const bool transB = (opB == OP_T || opB == OP_C), conjB = (opB == OP_C || opB == OP_R);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tiles = (M + kSkinnyRows - 1) / kSkinnyRows;
  for (int64_t job = blockIdx.x; job < tiles * batch; job += gridDim.x) {
    const int64_t bz = job / tiles, i0 = (job % tiles) * kSkinnyRows;
    const T* Bb = B + bz * sB;
    const T* Ab = A + bz * sA;
    __syncthreads();  // the previous job's readers are done
    if (warp == 0) {
      int base = 0;
      for (int j = 0; j < N; ++j) {
        T v;
        zero(v);
        if (lane < K) v = ld(transB ? Bb + j + (int64_t)lane * ldb : Bb + lane + (int64_t)j * ldb, conjB);
        const unsigned m = __ballot_sync(0xffffffffu, nonzero(v));
        if (lane == 0) colptr[j] = base;
        if (nonzero(v)) {
          const int pos = base + __popc(m & ((1u << lane) - 1u));
          nzv[pos] = v;
          nzk[pos] = (unsigned char)lane;
        }
        base += __popc(m);
      }
      if (lane == 0) colptr[N] = base;
    }
    const int64_t i = i0 + tid;
    for (int k = 0; k < K; ++k) {
      T a;
      zero(a);
      if (i < M) a = ld(Ab + i + (int64_t)k * lda, conjA);
      As[k * kSkinnyRows + tid] = a;
    }
    __syncthreads();
    if (i < M) {
      T* Cb = C + bz * sC + i;
      for (int j = 0; j < N; ++j) {
        T acc;
        zero(acc);
        for (int t = colptr[j]; t < colptr[j + 1]; ++t) mac(acc, As[nzk[t] * kSkinnyRows + tid], nzv[t]);
        T* cp = Cb + (int64_t)j * ldc;
        *cp = sc.epi(acc, cp);
      }
    }
  }
}

void raise_smem_limit_gemm(const void* fn, int bytes) { ensure_smem_limit(fn, bytes); }

}  // namespace

void gemm_f64_simt(nsg_ctx* c, const GemmArgs& g) {
  if (g.M == 0 || g.N == 0 || g.batch == 0) return;
  if (g.N <= 32 && g.K <= 32 && g.K >= 1 && (g.opA == OP_N || g.opA == OP_R)) {
    const int64_t sms = c->num_sms > 0 ? c->num_sms : 152;
    const int64_t jobs = ((g.M + kSkinnyRows - 1) / kSkinnyRows) * g.batch;
    const int grid = int(std::min<int64_t>(jobs, sms * 16));
    ProfScope ps(c, NSG_PROF_SIMT_GEMM,
                 double(g.M) * double(g.N) * double(g.K) * double(g.batch) * (g.dtype == NSG_C128 ? 8.0 : 2.0));
    if (g.dtype == NSG_C128) {
      const int shm = int(g.K) * kSkinnyRows * 16;
      Scal<double2> sc{make_double2(g.alpha_re, g.alpha_im), make_double2(g.beta_re, g.beta_im)};
      raise_smem_limit_gemm((const void*)gemm_skinny_kernel<double2>, 32 * kSkinnyRows * 16);
      gemm_skinny_kernel<double2><<<grid, kSkinnyRows, shm, c->stream>>>(
          g.M, int(g.N), int(g.K), (const double2*)g.A, g.lda, g.strideA, g.opA == OP_R, (const double2*)g.B,
          g.ldb, g.strideB, g.opB, (double2*)g.C, g.ldc, g.strideC, g.batch, sc);
    } else {
      const int shm = int(g.K) * kSkinnyRows * 8;
      Scal<double> sc{g.alpha_re, g.beta_re};
      raise_smem_limit_gemm((const void*)gemm_skinny_kernel<double>, 32 * kSkinnyRows * 8);
      gemm_skinny_kernel<double><<<grid, kSkinnyRows, shm, c->stream>>>(
          g.M, int(g.N), int(g.K), (const double*)g.A, g.lda, g.strideA, false, (const double*)g.B, g.ldb,
          g.strideB, g.opB, (double*)g.C, g.ldc, g.strideC, g.batch, sc);
    }
    count_launch(c);
    check_launch("gemm_skinny");
    return;
  }
  int64_t gx = (g.M + BM - 1) / BM, gy = (g.N + BN - 1) / BN;
  NSG_CHECK(gx < (1ll << 31) && gy < 65536, NSG_ERR_UNSUPPORTED, "gemm: grid too large");
  // split K when the tile grid cannot fill the GPU
  int splits = 1;
  int64_t ksplit = g.K;
  const int64_t tiles = gx * gy * g.batch;
  const int64_t sms = c->num_sms > 0 ? c->num_sms : 152;
  if (tiles < sms && g.K >= 64) {
    // small outputs (the eigensolver's GEMMs at bond dimension <= 128 have a handful of
    // tiles): spread K over more SMs, down to 32-deep slices; the FP64 pipe of one SM is
    // the bound otherwise
    int64_t want = (2 * sms + tiles - 1) / tiles;
    int64_t maxs = g.K >= 512 ? g.K / 256 : g.K / 32;
    splits = int(std::min<int64_t>({want, maxs, 64}));
    if (splits < 2) splits = 1;
    ksplit = (g.K + splits - 1) / splits;
    ksplit = ((ksplit + 15) / 16) * 16;
    splits = int((g.K + ksplit - 1) / ksplit);
  }
  // the tuning table (or the context's override) replaces the rule for its buckets
  int tuned = c->tune_splitk;
  if (tuned == 0)
    for (const auto& t : tuning::kSplit)
      if (t.splits > 0 && tiles <= t.max_tiles && g.K <= t.max_k) {
        tuned = t.splits;
        break;
      }
  if (tuned > 0) {
    splits = int(std::min<int64_t>(tuned, std::max<int64_t>(1, g.K / 16)));
    ksplit = (g.K + splits - 1) / splits;
    ksplit = ((ksplit + 15) / 16) * 16;
    splits = int((g.K + ksplit - 1) / ksplit);
  }
  int64_t zt = g.batch * splits;
  int64_t gz = zt < 65535 ? zt : 65535;
  dim3 grid{unsigned(gx), unsigned(gy), unsigned(gz)};
  const size_t eb = g.dtype == NSG_C128 ? 16 : 8;
  ProfScope ps(c, NSG_PROF_SIMT_GEMM,
               double(g.M) * double(g.N) * double(g.K) * double(g.batch) * (g.dtype == NSG_C128 ? 8.0 : 2.0));
  void* W = nullptr;
  size_t wbytes = 0;
  void* Cout = g.C;
  if (splits > 1) {
    wbytes = eb * size_t(g.M) * size_t(g.N) * size_t(zt);
    W = dalloc(c, wbytes);
    Cout = W;
  }
  if (g.dtype == NSG_C128) {
    Scal<double2> sc{make_double2(g.alpha_re, g.alpha_im), make_double2(g.beta_re, g.beta_im)};
    gemm_kernel<double2, 8><<<grid, NT, 0, c->stream>>>(g.M, g.N, g.K, (const double2*)g.A, g.lda, g.strideA, g.opA,
                                                        (const double2*)g.B, g.ldb, g.strideB, g.opB,
                                                        (double2*)Cout, g.ldc, g.strideC, g.batch, sc, splits, ksplit);
    if (splits > 1) {
      int64_t tot = g.M * g.N * g.batch;
      int rb = int(std::min<int64_t>((tot + 255) / 256, sms * 8));
      splitk_reduce_kernel<double2><<<rb, 256, 0, c->stream>>>(g.M, g.N, g.batch, splits, (const double2*)W,
                                                              (double2*)g.C, g.ldc, g.strideC, sc);
      count_launch(c);
    }
  } else {
    Scal<double> sc{g.alpha_re, g.beta_re};
    gemm_kernel<double, 16><<<grid, NT, 0, c->stream>>>(g.M, g.N, g.K, (const double*)g.A, g.lda, g.strideA, g.opA,
                                                        (const double*)g.B, g.ldb, g.strideB, g.opB, (double*)Cout,
                                                        g.ldc, g.strideC, g.batch, sc, splits, ksplit);
    if (splits > 1) {
      int64_t tot = g.M * g.N * g.batch;
      int rb = int(std::min<int64_t>((tot + 255) / 256, sms * 8));
      splitk_reduce_kernel<double><<<rb, 256, 0, c->stream>>>(g.M, g.N, g.batch, splits, (const double*)W,
                                                             (double*)g.C, g.ldc, g.strideC, sc);
      count_launch(c);
    }
  }
  if (W) dfree(c, W, wbytes);
  count_launch(c);
  check_launch("gemm_f64_simt");
}

// FP64-level products: the eight-slice Ozaki tensor-core form (2^-55 of the row and
// column scales) when the split precision is selected, otherwise the FP64 CUDA cores
// (never TF32x3).
void gemm_accurate(nsg_ctx* c, const GemmArgs& g_in) {
  GemmArgs g = g_in;
  if (g.dtype == NSG_F64) {
    if (g.opA == OP_C) g.opA = OP_T;
    if (g.opA == OP_R) g.opA = OP_N;
    if (g.opB == OP_C) g.opB = OP_T;
    if (g.opB == OP_R) g.opB = OP_N;
  }
  if ((c->precision == NSG_PREC_OZAKI || c->precision == NSG_PREC_OZAKI8) && gemm_ozaki_tc(c, g, 8)) return;
  gemm_f64_simt(c, g);
}

void gemm(nsg_ctx* c, const GemmArgs& g_in) {
  GemmArgs g = g_in;
  if (g.dtype == NSG_F64) {  // conjugation is the identity on real data
    if (g.opA == OP_C) g.opA = OP_T;
    if (g.opA == OP_R) g.opA = OP_N;
    if (g.opB == OP_C) g.opB = OP_T;
    if (g.opB == OP_R) g.opB = OP_N;
  }
  double mac = double(g.M) * double(g.N) * double(g.K) * double(g.batch);
  c->flops += uint64_t(mac * (g.dtype == NSG_C128 ? 8.0 : 2.0));
  if (g.K == 0) {
    // C = beta*C (alpha term vanishes)
    return;
  }
  if (c->precision == NSG_PREC_TF32X3 && gemm_split_tc(c, g)) return;
  if (c->precision == NSG_PREC_OZAKI && gemm_ozaki_tc(c, g, 6)) return;
  if (c->precision == NSG_PREC_OZAKI8 && gemm_ozaki_tc(c, g, 8)) return;
  gemm_f64_simt(c, g);
}

}  // namespace nsg
