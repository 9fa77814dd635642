// FP64-accurate GEMM on the BF16 tensor cores by exact multi-slice splitting
// (the Ozaki scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012)).
//
// Row i of A is scaled by sigma_i = 2^ceil(log2 max_k |A_ik|) and written as
//   A_ik / sigma_i = sum_{s<S} 2^{-7(s+1)} A^(s)_ik + r,  A^(s) integers, |A^(s)| <= 128,
// (round-to-nearest digits, |r| <= 2^{-7S-1}); columns of B likewise with tau_j.  Then
//   (AB)_ij = sigma_i tau_j sum_g 2^{-7(g+2)} sum_{s+t=g} (A^(s) B^(t))_ij,   g <= S-1.
// The integer slices are exact in BF16, and with g+1 <= 6 products per group and K
// chunks of 128 every partial sum is an integer below 2^24, so the tcgen05 FP32
// accumulation of a group over a chunk is exact.  Drain warps add the six group sums
// of each chunk into double-float (hi, lo) FP32 accumulators; the epilogue widens to
// FP64 and applies sigma_i tau_j, alpha and beta.  With S = 6 slices the result is
// within ~2^-43 K sigma_i tau_j of A B (dropped slices and products).
//
// Kernel layout: 128 x 64 output tile per CTA, 16 drain warps (4 warpgroups, each
// owning 16 accumulator columns) + 1 TMA/MMA warp; three-stage ring of 32-wide K slabs
// holding all six slices of A and B (SWIZZLE_64B); 6 x 64 TMEM accumulator columns.
// All mbarrier waits are bounded; on time-out the CTA raises the error flag, drains its
// TMA copies (bounded), frees its TMEM and returns.
#include "nsg_internal.h"

#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

namespace nsg {

namespace {

constexpr int BM = 128, BN = 64, BKS = 32;  // K slab: 32 bf16 = 64 bytes
constexpr int SLICE_A = BM * BKS * 2;       // 8 KB
constexpr int SLICE_B = BN * BKS * 2;       // 4 KB
constexpr int CHUNK_SLABS = 4;              // K = 128 per exact chunk
constexpr int NDRAIN_WARPS = 16;
constexpr int NTHREADS = (NDRAIN_WARPS + 1) * 32;

// S slices per operand, groups g = s + t in [0, S-1] (G x 64 TMEM columns <= 512);
// S = 8 fills TMEM and leaves room for two 96 KB stages of shared memory.
template <int S_>
struct Oz {
  static constexpr int S = S_, G = S_;
  static constexpr int STAGES = S_ <= 6 ? 3 : 2;
  static constexpr int STAGE_BYTES = S * (SLICE_A + SLICE_B);
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512;
  static_assert(G * BN <= 512, "accumulators exceed TMEM");
  static_assert(SMEM_BYTES <= 227 * 1024, "stages exceed shared memory");
};
constexpr long long kWaitLimit = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* fail) {
  for (long long i = 0; i < kWaitLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (fail && *fail) return false;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
// K-major operand, 64-byte swizzle: 8-row groups 512 bytes apart
__device__ __forceinline__ uint64_t sdesc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)((512u >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)4u << 61;  // 64-byte swizzle
  return d;
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---------------------------------------------------------------------------
// scales: scale[b][r] = 2^ceil(log2 max_k |src(r, k)|) (1 for an all-zero row)
// ---------------------------------------------------------------------------
__global__ void row_scale_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t rs, int64_t ks,
                                 int64_t bs, int64_t rows_p, double* __restrict__ scale, int64_t batch) {
  // one warp per row; lanes stride over k
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = (gridDim.x * (int64_t)blockDim.x) >> 5;
  for (int64_t t = w; t < rows_p * batch; t += nw) {
    int64_t r = t % rows_p, b = t / rows_p;
    double m = 0.0;
    if (r < rows) {
      const double* base = src + b * bs + r * rs;
      for (int64_t k = lane; k < K; k += 32) m = fmax(m, fabs(base[k * ks]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
      int e = 0;
      if (m > 0) {
        frexp(m, &e);  // m = f 2^e, f in [0.5, 1)  ->  m <= 2^e
      }
      // a normal power of two (the slicer inverts it by exponent arithmetic)
      scale[t] = (m > 0) ? ldexp(1.0, max(e, -1000)) : 1.0;
    }
  }
}

// slices: out[(b*S + s)][r][k] (bf16, K-major, padded with zeros)
template <int S>
__global__ void slice_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t rs, int64_t ks,
                             int64_t bs, int64_t rows_p, int64_t K_p, const double* __restrict__ scale,
                             __nv_bfloat16* __restrict__ out, int64_t batch) {
  __shared__ double tile[32][33];
  const int64_t tr = rows_p / 32, tk = K_p / 32;
  const int64_t ntiles = tr * tk * batch;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int64_t kt = t % tk, rt = (t / tk) % tr, b = t / (tk * tr);
    const double* base = src + b * bs;
    if (ks == 1) {
      for (int i = ty; i < 32; i += 8) {
        int64_t r = rt * 32 + i, k = kt * 32 + tx;
        tile[i][tx] = (r < rows && k < K) ? base[r * rs + k] : 0.0;
      }
    } else {
      for (int j = ty; j < 32; j += 8) {
        int64_t r = rt * 32 + tx, k = kt * 32 + j;
        tile[tx][j] = (r < rows && k < K) ? base[r * rs + k * ks] : 0.0;
      }
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
      int64_t r = rt * 32 + i, k = kt * 32 + tx;
      // x = value / sigma_r in [-1, 1] (sigma_r a power of two: the product is exact),
      // then X = round(x 2^{7S}) in int64 and balanced 7-bit digits of X peeled off from
      // the top with integer shifts (round half up): X = sum_s d_s 2^{7(S-1-s)}, |d_0| <=
      // 128, |d_s| <= 64 after it, and |x - X 2^{-7S}| <= 2^{-7S-1}.  Only one FP64
      // multiply and one conversion per element: the FP64 pipe is the slow one here.
      // 1 / sigma_r by exponent arithmetic (sigma_r is a normal power of two)
      const double inv = __longlong_as_double(0x7FE0000000000000ll - __double_as_longlong(scale[b * rows_p + r]));
      constexpr double kFix = double(1ull << (7 * S));
      long long X = __double2ll_rn(tile[i][tx] * inv * kFix);
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int sh = 7 * (S - 1 - s);
        const long long dgt = sh ? ((X + (1ll << (sh - 1))) >> sh) : X;
        X -= dgt << sh;
        size_t o = ((size_t)(b * S + s) * rows_p + r) * K_p + k;
        out[o] = __float2bfloat16_rn((float)(int)dgt);  // |dgt| <= 128: exact in bf16
      }
    }
    __syncthreads();
  }
}

struct OzEpi {
  double* C;
  int64_t ldc, sC, M, N;
  int64_t crs;  // stride between rows of C in doubles (1, or 2 for one part of complex C)
  double alpha, beta;
  const double* sa;  // row scales of A  [batch_a][Mp]
  const double* sb;  // row scales of B^T [batch_b][Np]
  int64_t Mp, Np;
  int a_batched, b_batched;
  int* err;
  // split K: grid z = batch x nsplit, split s takes K slabs [s split_slabs, ..) (whole
  // exact chunks) and writes its scaled partial product to W[z] (M x N, column-major);
  // oz_split_reduce_kernel adds the splits in order and applies alpha and beta
  int nsplit, split_slabs;
  double* W;
};

// float -> double by exponent re-bias (exact for normal floats; zero, subnormals, inf and
// NaN take the conversion instruction)
__device__ __forceinline__ double widen(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;
  const uint64_t d = ((uint64_t)(b >> 31) << 63) | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}
// exponent k of a normal power of two 2^k
__device__ __forceinline__ int pow2_exponent(double p) {
  return int((__double_as_longlong(p) >> 52) & 0x7FF) - 1023;
}
// v * 2^k by adding k to the exponent field when the result stays normal
__device__ __forceinline__ double scale_pow2(double v, int k) {
  const long long b = __double_as_longlong(v);
  const int e = int((b >> 52) & 0x7FF);
  if (e == 0 || e == 0x7FF || e + k <= 0 || e + k >= 0x7FF) return v * ldexp(1.0, k);
  return __longlong_as_double(b + ((long long)k << 52));
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  float s = hi + x;
  float bb = s - hi;
  float e = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += e;
}

template <int S_>
__global__ void __launch_bounds__(NTHREADS, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int nk,
                   OzEpi ep) {
  constexpr int S = Oz<S_>::S, G = Oz<S_>::G, STAGES = Oz<S_>::STAGES, STAGE_BYTES = Oz<S_>::STAGE_BYTES;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accfull = empty + STAGES;
  uint64_t* accempty = accfull + 1;
  uint32_t* tmem_slot = (uint32_t*)(accempty + 1);
  volatile int* fail = (volatile int*)(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int sp = int(blockIdx.z % unsigned(ep.nsplit)), bz = int(blockIdx.z / unsigned(ep.nsplit));
  const int tb = sp * ep.split_slabs;           // this split's first K slab (global index)
  const int nkl = min(nk - tb, ep.split_slabs);  // its slabs; the pipeline counts from 0
  const int nchunks = (nkl + CHUNK_SLABS - 1) / CHUNK_SLABS;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accfull, 1);
    mbar_init(accempty, NDRAIN_WARPS * 32);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == NDRAIN_WARPS) {
    if (lane == 0) {
      // kind::f16: D F32 (bits 4-5 = 1), A BF16 (7-9 = 1), B BF16 (10-12 = 1), K-major both
      // instruction descriptor for an N-wide product (N = 64 .. 256, a multiple of 64 here)
      const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BM >> 4) << 24);
      auto idesc_n = [&](int n) { return idesc0 | ((uint32_t)(n >> 3) << 17); };
      auto a_ptr = [&](int st, int s) { return smem + st * STAGE_BYTES + s * SLICE_A; };
      auto b_ptr = [&](int st, int s) { return smem + st * STAGE_BYTES + S * SLICE_A + s * SLICE_B; };
      auto issue = [&](int t, int st) {
        mbar_expect_tx(&full[st], STAGE_BYTES);
        const int kc = (tb + t) * BKS;
        tma_load_3d(a_ptr(st, 0), &mapA, &full[st], kc, m0, (ep.a_batched ? bz : 0) * S);
        tma_load_3d(b_ptr(st, 0), &mapB, &full[st], kc, n0, (ep.b_batched ? bz : 0) * S);
      };
      const int pre = nkl < STAGES ? nkl : STAGES;
      for (int t = 0; t < pre; ++t) issue(t, t);
      int issued = pre;
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        if (c >= 1 && !mbar_wait(accempty, (c - 1) & 1, fail)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int t0 = c * CHUNK_SLABS, t1 = min(nkl, t0 + CHUNK_SLABS);
        for (int t = t0; t < t1 && ok; ++t) {
          const int st = t % STAGES;
          if (!mbar_wait(&full[st], (t / STAGES) & 1, fail)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
          for (int kk = 0; kk < BKS / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 = 32 bytes inside the 64-byte swizzle atom
            // A^(s) meets B^(0..G-1-s) in one product of width (G-s) x BN: the B slices lie
            // back to back along N in shared memory (8-row groups 512 B apart throughout)
            // and the accumulators of groups s .. G-1 back to back in TMEM, so D columns
            // [s BN, G BN) += A^(s) [B^(0) | ... | B^(G-1-s)], split in widths <= 256.
            // (One 64-wide product per slice pair re-read A from shared memory 21 times.)
#pragma unroll
            for (int sa = 0; sa < S; ++sa) {
              const uint64_t ad = sdesc64(smem_u32(a_ptr(st, sa)) + off);
#pragma unroll
              for (int u0 = 0; u0 < G - sa; u0 += 4) {
                const int width = (G - sa - u0) >= 4 ? 4 * BN : (G - sa - u0) * BN;
                // every accumulator's first product of the chunk is the sa = 0 one at t0, kk 0
                mma_bf16(tmem + (uint32_t)((sa + u0) * BN), ad, sdesc64(smem_u32(b_ptr(st, u0)) + off),
                         idesc_n(width), (t == t0 && kk == 0 && sa == 0) ? 0u : 1u);
              }
            }
          }
          mma_commit(&empty[st]);
          if (t >= 1 && issued < nkl) {
            const int sp = (t - 1) % STAGES;
            if (!mbar_wait(&empty[sp], ((t - 1) / STAGES) & 1, fail)) {
              ok = false;
              break;
            }
            issue(issued, sp);
            ++issued;
          }
        }
        if (!ok) break;
        mma_commit(accfull);
      }
      if (!ok) {
        *fail = 1;
        atomicExch(ep.err, 1);
        for (int t = 0; t < issued; ++t) mbar_wait(&full[t % STAGES], (t / STAGES) & 1, nullptr);
      }
    }
  } else {
    // drain warps: warpgroup q = warp / 4 owns columns [16 q, 16 q + 16); TMEM lanes 32 (warp % 4) ..
    const int q = warp >> 2, wl = warp & 3;
    float hi[16], lo[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) hi[j] = lo[j] = 0.f;
    const uint32_t lane_base = (uint32_t)(wl * 32) << 16;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      if (!mbar_wait(accfull, c & 1, fail)) {
        ok = false;
        atomicExch(ep.err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // three groups' TMEM loads in flight per wait (one wait per group made the drain,
      // and with it the tensor pipe, wait on the load latency six times per chunk); the
      // groups are still added in ascending order
#pragma unroll
      for (int g0 = 0; g0 < G; g0 += 3) {
        uint32_t r[3][16];
#pragma unroll
        for (int gg = 0; gg < 3; ++gg) {
          if (g0 + gg < G)
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15}, [%16];"
                : "=r"(r[gg][0]), "=r"(r[gg][1]), "=r"(r[gg][2]), "=r"(r[gg][3]), "=r"(r[gg][4]), "=r"(r[gg][5]),
                  "=r"(r[gg][6]), "=r"(r[gg][7]), "=r"(r[gg][8]), "=r"(r[gg][9]), "=r"(r[gg][10]), "=r"(r[gg][11]),
                  "=r"(r[gg][12]), "=r"(r[gg][13]), "=r"(r[gg][14]), "=r"(r[gg][15])
                : "r"(tmem + lane_base + (uint32_t)((g0 + gg) * BN + 16 * q)));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (g0 + 3 >= G) {
          // the last loads are in registers: release the accumulators before the
          // arithmetic, so the next chunk's products overlap it
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          mbar_arrive(accempty);
        }
#pragma unroll
        for (int gg = 0; gg < 3; ++gg) {
          if (g0 + gg < G) {
            const float sc = __int_as_float((127 - 7 * (g0 + gg + 2)) << 23);  // 2^{-7(g+2)}, exact
#pragma unroll
            for (int j = 0; j < 16; ++j) two_sum_acc(hi[j], lo[j], __uint_as_float(r[gg][j]) * sc);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {  // renormalise (fast two-sum)
        float s = hi[j] + lo[j];
        lo[j] = lo[j] - (s - hi[j]);
        hi[j] = s;
      }
    }
    if (ok) {
      // Epilogue with as few FP64-pipe operations as possible (GB300 runs FP64 at ~2 per
      // clock per SM, and this loop touches every output): the FP32 pair is widened by
      // exponent arithmetic, added with one DADD, and the power-of-two scales sigma_i tau_j
      // are applied to the exponent field; alpha = 1 costs nothing further.
      const int64_t row = m0 + wl * 32 + lane;
      if (row < ep.M) {
        const int ka = pow2_exponent(ep.sa[(ep.a_batched ? bz : 0) * ep.Mp + row]);
        const bool unit_alpha = ep.alpha == 1.0;
        double* Wz = ep.nsplit > 1 ? ep.W + (size_t)blockIdx.z * ep.M * ep.N : nullptr;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t col = n0 + 16 * q + j;
          if (col < ep.N) {
            const int kb = pow2_exponent(ep.sb[(ep.b_batched ? bz : 0) * ep.Np + col]);
            double v = scale_pow2(widen(hi[j]) + widen(lo[j]), ka + kb);
            if (Wz) {
              Wz[row + col * ep.M] = v;
            } else {
              if (!unit_alpha) v *= ep.alpha;
              double* cp = ep.C + bz * ep.sC + row * ep.crs + col * ep.ldc;
              *cp = (ep.beta == 0.0) ? v : fma(ep.beta, *cp, v);
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// C = alpha sum_s W[b nsplit + s] + beta C, the splits added in order
__global__ void oz_split_reduce_kernel(const double* __restrict__ W, int nsplit, int64_t M, int64_t N,
                                       int64_t batch, double* __restrict__ C, int64_t ldc, int64_t sC, int64_t crs,
                                       double alpha, double beta) {
  const int64_t MN = M * N, tot = MN * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / MN, r = e - b * MN, row = r % M, col = r / M;
    double acc = 0.0;
    for (int sp = 0; sp < nsplit; ++sp) acc += W[(b * nsplit + sp) * MN + r];
    const double v = alpha == 1.0 ? acc : acc * alpha;
    double* cp = C + b * sC + row * crs + col * ldc;
    *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
  }
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeFn)p;
  });
  return fn;
}

// slices [planes = batch*S][rows_p][K_p] bf16; box {32, box_rows, S}
CUtensorMap make_map(void* base, int64_t rows_p, int64_t K_p, int64_t planes, int box_rows, int S) {
  EncodeFn enc = encode_fn();
  NSG_CHECK(enc != nullptr, NSG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)K_p, (cuuint64_t)rows_p, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(K_p * 2), (cuuint64_t)(K_p * rows_p * 2)};
  cuuint32_t box[3] = {(cuuint32_t)BKS, (cuuint32_t)box_rows, (cuuint32_t)S};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  NSG_CHECK(r == CUDA_SUCCESS, NSG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

template <int S>
void slice_operand(nsg_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, int64_t ks, int64_t bs,
                   int64_t batch, int64_t rows_p, int64_t K_p, double* scale, __nv_bfloat16* out) {
  {
    int64_t warps = rows_p * batch;
    int grid = int(std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)c->num_sms * 16));
    ProfScope ps(c, NSG_PROF_SPLIT, 0.0);
    row_scale_kernel<<<grid, 256, 0, c->stream>>>(src, rows, K, rs, ks, bs, rows_p, scale, batch);
  }
  int64_t ntiles = (rows_p / 32) * (K_p / 32) * batch;
  int grid = int(std::min<int64_t>(ntiles, (int64_t)c->num_sms * 16));
  ProfScope ps(c, NSG_PROF_SPLIT, 0.0);
  slice_kernel<S><<<grid, 256, 0, c->stream>>>(src, rows, K, rs, ks, bs, rows_p, K_p, scale, out, batch);
  count_launch(c, 2);
  check_launch("ozaki slices");
}

// One operand of an Ozaki product, sliced: S bf16 slices [batch][S][rows_p][K_p] and the
// power-of-two row scales [batch][rows_p].
struct OzOperand {
  __nv_bfloat16* slices = nullptr;
  double* scales = nullptr;
  int64_t rows_p = 0, batch = 1;
};

template <int S>
size_t oz_operand_bytes(int64_t rows_p, int64_t K_p, int64_t batch) {
  return ((2 * size_t(S) * rows_p * K_p * batch + 255) & ~size_t(255)) + ((8 * size_t(rows_p) * batch + 255) & ~size_t(255));
}

// slices of op(X) viewed as rows x K (element (r, k) at src[b bs + r rs + k ks], in doubles)
template <int S>
OzOperand oz_prepare(nsg_ctx* c, unsigned char* mem, const double* src, int64_t rows, int64_t K, int64_t rs,
                     int64_t ks, int64_t bs, int64_t batch, int64_t rows_p, int64_t K_p) {
  OzOperand o;
  o.slices = (__nv_bfloat16*)mem;
  o.scales = (double*)(mem + ((2 * size_t(S) * rows_p * K_p * batch + 255) & ~size_t(255)));
  o.rows_p = rows_p;
  o.batch = batch;
  slice_operand<S>(c, src, rows, K, rs, ks, bs, batch, rows_p, K_p, o.scales, o.slices);
  return o;
}

// C (+)= alpha A B^T-form product of two prepared operands into C (stride ldc between
// columns, sC between batch entries, crs between rows; all in doubles)
template <int S>
void oz_product(nsg_ctx* c, const OzOperand& A, const OzOperand& B, int64_t M, int64_t N, int64_t K_p, int64_t batch,
                double* C, int64_t ldc, int64_t sC, int64_t crs, double alpha, double beta, int64_t flop_k) {
  constexpr int SMEM_BYTES = Oz<S>::SMEM_BYTES;
  CUtensorMap mA = make_map(A.slices, A.rows_p, K_p, S * A.batch, BM, S),
              mB = make_map(B.slices, B.rows_p, K_p, S * B.batch, BN, S);
  int* err = device_flag(c);  // checked once at the end of the public call
  ensure_smem_limit((const void*)oz_gemm_kernel<S>, SMEM_BYTES);
  // split K over whole exact chunks when the output tiles would leave most SMs idle
  // (the small products of a converged sweep: 32-64 tiles of 128 x 64 on 152 SMs)
  const int nk = int(K_p / BKS), nchunk = (nk + CHUNK_SLABS - 1) / CHUNK_SLABS;
  const int64_t tiles = (A.rows_p / BM) * (B.rows_p / BN) * batch;
  const int64_t sms = c->num_sms > 0 ? c->num_sms : 152;
  int nsplit = 1;
  if (tiles * 2 <= sms && nchunk >= 2)
    nsplit = int(std::min<int64_t>({(int64_t)nchunk, sms / tiles, 16, 65535 / batch}));
  const int split_slabs = (nchunk + nsplit - 1) / nsplit * CHUNK_SLABS;
  nsplit = (nk + split_slabs - 1) / split_slabs;
  // the partial products' workspace, only when K is split (freed on every exit)
  struct Partials {
    nsg_ctx* c;
    void* p;
    size_t bytes;
    ~Partials() {
      try {
        dfree(c, p, bytes);
      } catch (...) {
      }
    }
  } wbuf{c, nullptr, 0};
  if (nsplit > 1) {
    wbuf.bytes = sizeof(double) * size_t(nsplit) * size_t(batch) * size_t(M) * size_t(N);
    wbuf.p = dalloc(c, wbuf.bytes);
  }
  OzEpi ep{C,        ldc,         sC,          M,     N,     crs,  alpha, beta, A.scales, B.scales, A.rows_p, B.rows_p,
           A.batch > 1, B.batch > 1, err, nsplit, split_slabs, (double*)wbuf.p};
  dim3 grid(unsigned(A.rows_p / BM), unsigned(B.rows_p / BN), unsigned(batch * nsplit));
  {
    ProfScope ps(c, NSG_PROF_TC_GEMM, 2.0 * double(M) * double(N) * double(flop_k) * double(batch));
    oz_gemm_kernel<S><<<grid, NTHREADS, SMEM_BYTES, c->stream>>>(mA, mB, nk, ep);
    if (nsplit > 1) {
      const int64_t tot = M * N * batch;
      const int rg = int(std::min<int64_t>((tot + 255) / 256, sms * 8));
      oz_split_reduce_kernel<<<rg, 256, 0, c->stream>>>((const double*)wbuf.p, nsplit, M, N, batch, C, ldc, sC, crs,
                                                        alpha, beta);
    }
  }
  count_launch(c, nsplit > 1 ? 2 : 1);
  check_launch("oz_gemm");
}

template <int S>
bool gemm_ozaki_impl(nsg_ctx* c, const GemmArgs& g) {
  if (g.dtype != NSG_F64 && g.dtype != NSG_C128) return false;
  if (g.M < 64 || g.N < 32 || g.K < 64) return false;
  if (g.batch > 65535) return false;
  const bool cplx = g.dtype == NSG_C128;
  if (!cplx && (g.opA == OP_C || g.opA == OP_R || g.opB == OP_C || g.opB == OP_R)) return false;
  // complex: real scalars only (the four real products carry the signs)
  if (cplx && (g.alpha_im != 0.0 || g.beta_im != 0.0)) return false;
  const int64_t Mp = (g.M + BM - 1) / BM * BM, Np = (g.N + BN - 1) / BN * BN, Kp = (g.K + BKS - 1) / BKS * BKS;
  const bool transA = g.opA == OP_T || g.opA == OP_C, transB = g.opB == OP_T || g.opB == OP_C;
  const int64_t ars = !transA ? 1 : g.lda, aks = !transA ? g.lda : 1;
  const int64_t brs = !transB ? g.ldb : 1, bks = !transB ? 1 : g.ldb;
  const int64_t ab = (g.strideA == 0) ? 1 : g.batch, bb = (g.strideB == 0) ? 1 : g.batch;
  const size_t opA_bytes = oz_operand_bytes<S>(Mp, Kp, ab), opB_bytes = oz_operand_bytes<S>(Np, Kp, bb);
  if (!cplx) {
    ScopedBuf sbuf(c, opA_bytes + opB_bytes);
    unsigned char* buf = (unsigned char*)sbuf.p;
    OzOperand A = oz_prepare<S>(c, buf, (const double*)g.A, g.M, g.K, ars, aks, g.strideA, ab, Mp, Kp);
    OzOperand B = oz_prepare<S>(c, buf + opA_bytes, (const double*)g.B, g.N, g.K, brs, bks, g.strideB, bb, Np, Kp);
    oz_product<S>(c, A, B, g.M, g.N, Kp, g.batch, (double*)g.C, g.ldc, g.strideC, 1, g.alpha_re, g.beta_re, g.K);
    return true;
  }
  // complex: A = Ar + i sa Ai, B = Br + i sb Bi (sa, sb = -1 for conjugated operands), as
  // four real products on the interleaved parts (strides doubled, imaginary parts at +1):
  //   Re C = alpha (Ar Br - sa sb Ai Bi) + beta Re C,  Im C = alpha (sb Ar Bi + sa Ai Br) + beta Im C
  const double sa = (g.opA == OP_C || g.opA == OP_R) ? -1.0 : 1.0;
  const double sbs = (g.opB == OP_C || g.opB == OP_R) ? -1.0 : 1.0;
  ScopedBuf sbuf(c, 2 * (opA_bytes + opB_bytes));
  unsigned char* buf = (unsigned char*)sbuf.p;
  const double* Ad = (const double*)g.A;
  const double* Bd = (const double*)g.B;
  OzOperand Ar = oz_prepare<S>(c, buf, Ad, g.M, g.K, 2 * ars, 2 * aks, 2 * g.strideA, ab, Mp, Kp);
  OzOperand Ai = oz_prepare<S>(c, buf + opA_bytes, Ad + 1, g.M, g.K, 2 * ars, 2 * aks, 2 * g.strideA, ab, Mp, Kp);
  OzOperand Br = oz_prepare<S>(c, buf + 2 * opA_bytes, Bd, g.N, g.K, 2 * brs, 2 * bks, 2 * g.strideB, bb, Np, Kp);
  OzOperand Bi = oz_prepare<S>(c, buf + 2 * opA_bytes + opB_bytes, Bd + 1, g.N, g.K, 2 * brs, 2 * bks,
                               2 * g.strideB, bb, Np, Kp);
  double* Cr = (double*)g.C;
  double* Ci = Cr + 1;
  const int64_t ldc = 2 * g.ldc, sC = 2 * g.strideC;
  const double al = g.alpha_re, be = g.beta_re;
  oz_product<S>(c, Ar, Br, g.M, g.N, Kp, g.batch, Cr, ldc, sC, 2, al, be, g.K);
  oz_product<S>(c, Ai, Bi, g.M, g.N, Kp, g.batch, Cr, ldc, sC, 2, -sa * sbs * al, 1.0, g.K);
  oz_product<S>(c, Ar, Bi, g.M, g.N, Kp, g.batch, Ci, ldc, sC, 2, sbs * al, be, g.K);
  oz_product<S>(c, Ai, Br, g.M, g.N, Kp, g.batch, Ci, ldc, sC, 2, sa * al, 1.0, g.K);
  return true;
}

}  // namespace

bool gemm_ozaki_tc(nsg_ctx* c, const GemmArgs& g, int slices) {
  if (slices == 8) return gemm_ozaki_impl<8>(c, g);
  return gemm_ozaki_impl<6>(c, g);
}

}  // namespace nsg
