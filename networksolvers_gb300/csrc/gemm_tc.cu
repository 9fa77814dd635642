// Split-precision FP64 GEMM on the tcgen05 tensor cores (sm_103a).
//
// C = alpha * op(A) op(B) + beta * C for real FP64 operands, computed as TF32x3:
// each operand x is split into TF32 slices x = hi + lo (hi = round_tf32(x),
// lo = round_tf32(x - hi)) and C ~= A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32
// accumulation in tensor memory; the epilogue widens to FP64.
//
//  * split pass: FP64 (any orientation, strided batch) -> two FP32 slice arrays in a
//    K-major, zero-padded layout [batch][rows_p][K_p] (rows_p % 128 == 0, K_p % 32 == 0),
//    through a 32 x 32 shared-memory transpose when the source is row-major in K.
//  * GEMM: one 128 x BN output tile per CTA; TMA (3-D tensor maps, 128-byte swizzle)
//    fills a 3-stage ring of {A_hi, A_lo, B_hi, B_lo} 32-wide K slabs; one thread
//    issues tcgen05.mma (kind::tf32, M=128, N=BN, K=8) four k-steps x three
//    products per slab and releases the slab with tcgen05.commit; 128 threads drain
//    the TMEM accumulator (tcgen05.ld 32x32b) into FP64.
//  * every mbarrier wait is bounded; on time-out the CTA raises the context's error
//    flag, drains its TMA copies (bounded), frees its TMEM and returns, and the host
//    reports NSG_ERR_TIMEOUT.
#include "nsg_internal.h"

#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <mutex>

namespace nsg {

namespace {

constexpr int TM = 128;      // tile rows (M)
constexpr int BN = 128;      // tile cols (N)
constexpr int BK = 32;       // K slab (32 fp32 = 128 bytes = one swizzle atom row)
constexpr int STAGES = 3;
constexpr int SLAB_A = TM * BK * 4;  // 16 KB
constexpr int SLAB_B = BN * BK * 4;  // 16 KB
constexpr int STAGE_BYTES = 2 * SLAB_A + 2 * SLAB_B;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr long long kWaitLimit = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;                     // leading byte offset (unused for this layout)
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;  // stride byte offset
  d |= (uint64_t)1u << 46;                     // descriptor version
  d |= (uint64_t)2u << 61;                     // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ---------------------------------------------------------------------------
// split pass: out_hi/out_lo[b][r][k] (K-major, padded) from src(r, k) = base[b*bs + r*rs + k*ks]
// ---------------------------------------------------------------------------
__global__ void split_tf32_kernel(const double* __restrict__ src, int64_t rows, int64_t K, int64_t rs, int64_t ks,
                                  int64_t bs, int64_t rows_p, int64_t K_p, float* __restrict__ hi,
                                  float* __restrict__ lo, int64_t batch) {
  __shared__ double tile[32][33];
  const int64_t tr = (rows_p + 31) / 32, tk = K_p / 32;
  const int64_t ntiles = tr * tk * batch;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int64_t kt = t % tk, rt = (t / tk) % tr, b = t / (tk * tr);
    const double* base = src + b * bs;
    // load a 32x32 tile with the contiguous source axis on the lanes
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
      if (r < rows_p) {
        double x = tile[i][tx];
        float h = tf32_round((float)x);
        float l = tf32_round((float)(x - (double)h));
        size_t o = (size_t)b * rows_p * K_p + (size_t)r * K_p + k;
        hi[o] = h;
        lo[o] = l;
      }
    }
    __syncthreads();
  }
}

struct EpiParams {
  double* C;
  int64_t ldc, sC;
  int64_t M, N;
  double alpha, beta;
  int* err;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 160 threads: warps 0-3 drain the accumulator (thread t owns output row m0 + t),
// warp 4 lane 0 issues TMA and MMA.  The K loop is cut into chunks of CH slabs; each
// chunk accumulates in one of two TMEM buffers and is added into FP32 registers by the
// drain warps (round-to-nearest adds), while the next chunk runs on the other buffer.
constexpr int CH = 2;                 // slabs per chunk (K = 64)
constexpr int NTHREADS = 160;

__global__ void __launch_bounds__(NTHREADS, 1)
    tc_gemm_tf32x3_kernel(const __grid_constant__ CUtensorMap mapAh, const __grid_constant__ CUtensorMap mapAl,
                          const __grid_constant__ CUtensorMap mapBh, const __grid_constant__ CUtensorMap mapBl,
                          int nk, EpiParams ep) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accfull = empty + STAGES;   // 2
  uint64_t* accempty = accfull + 2;     // 2
  uint32_t* tmem_slot = (uint32_t*)(accempty + 2);
  volatile int* fail = (volatile int*)(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * BN, bz = blockIdx.z;
  const int nchunks = (nk + CH - 1) / CH;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], 128);
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    if ((tid & 31) == 0) {
      const uint32_t idesc =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
      auto stage_ptr = [&](int s, int which) -> unsigned char* {
        return smem + s * STAGE_BYTES + (which < 2 ? which * SLAB_A : 2 * SLAB_A + (which - 2) * SLAB_B);
      };
      auto issue = [&](int t, int s) {
        mbar_expect_tx(&full[s], STAGE_BYTES);
        const int kc = t * BK;
        tma_load_3d(stage_ptr(s, 0), &mapAh, &full[s], kc, m0, bz);
        tma_load_3d(stage_ptr(s, 1), &mapAl, &full[s], kc, m0, bz);
        tma_load_3d(stage_ptr(s, 2), &mapBh, &full[s], kc, n0, bz);
        tma_load_3d(stage_ptr(s, 3), &mapBl, &full[s], kc, n0, bz);
      };
      const int pre = nk < STAGES ? nk : STAGES;
      for (int t = 0; t < pre; ++t) issue(t, t);
      int issued = pre;
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        const int buf = c & 1;
        if (c >= 2 && !mbar_wait(&accempty[buf], ((c >> 1) - 1) & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc_addr = tmem + (uint32_t)(buf * BN);
        const int t0 = c * CH, t1 = min(nk, t0 + CH);
        for (int t = t0; t < t1; ++t) {
          const int s = t % STAGES;
          if (!mbar_wait(&full[s], (t / STAGES) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t ah = smem_u32(stage_ptr(s, 0)), al = smem_u32(stage_ptr(s, 1));
          const uint32_t bh = smem_u32(stage_ptr(s, 2)), bl = smem_u32(stage_ptr(s, 3));
#pragma unroll
          for (int kk = 0; kk < BK / 8; ++kk) {
            const uint32_t off = kk * 32;  // 8 tf32 = 32 bytes inside the swizzle atom
            const uint32_t first = (t == t0 && kk == 0) ? 0u : 1u;
            mma_tf32(acc_addr, sdesc(ah + off), sdesc(bh + off), idesc, first);
            mma_tf32(acc_addr, sdesc(ah + off), sdesc(bl + off), idesc, 1u);
            mma_tf32(acc_addr, sdesc(al + off), sdesc(bh + off), idesc, 1u);
          }
          mma_commit(&empty[s]);
          if (t >= 1 && issued < nk) {
            const int sp = (t - 1) % STAGES;
            if (!mbar_wait(&empty[sp], ((t - 1) / STAGES) & 1)) {
              ok = false;
              break;
            }
            issue(issued, sp);
            ++issued;
          }
        }
        if (!ok) break;
        mma_commit(&accfull[buf]);
      }
      if (!ok) {
        *fail = 1;
        atomicExch(ep.err, 1);
        for (int t = 0; t < issued; ++t) mbar_wait(&full[t % STAGES], (t / STAGES) & 1);
      }
    }
  } else {
    // drain warps
    float sum[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) sum[j] = 0.f;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      const int buf = c & 1;
      bool got = false;
      for (long long i = 0; i < kWaitLimit && !got; ++i) {
        got = mbar_try_wait(&accfull[buf], (c >> 1) & 1);
        if (*fail) break;
      }
      if (!got) {
        ok = false;
        atomicExch(ep.err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c0 = 0; c0 < BN; c0 += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(tmem + lane_base + (uint32_t)(buf * BN + c0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[c0 + j] += __uint_as_float(r[j]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&accempty[buf]);
    }
    if (ok) {
      const int64_t row = m0 + tid;
      if (row < ep.M) {
#pragma unroll
        for (int j = 0; j < BN; ++j) {
          const int64_t col = n0 + j;
          if (col < ep.N) {
            double* cp = ep.C + bz * ep.sC + row + col * ep.ldc;
            const double v = (double)sum[j];
            *cp = (ep.beta == 0.0) ? ep.alpha * v : fma(ep.alpha, v, ep.beta * (*cp));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
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

CUtensorMap make_map(void* base, int64_t rows_p, int64_t K_p, int64_t batch, int box_rows) {
  EncodeFn enc = encode_fn();
  NSG_CHECK(enc != nullptr, NSG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)K_p, (cuuint64_t)rows_p, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)(K_p * 4), (cuuint64_t)(K_p * rows_p * 4)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  NSG_CHECK(r == CUDA_SUCCESS, NSG_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

void split_operand(nsg_ctx* c, const double* src, int64_t rows, int64_t K, int64_t rs, int64_t ks, int64_t bs,
                   int64_t batch, int64_t rows_p, int64_t K_p, float* hi, float* lo) {
  int64_t ntiles = ((rows_p + 31) / 32) * (K_p / 32) * batch;
  int grid = int(std::min<int64_t>(ntiles, (int64_t)c->num_sms * 16));
  ProfScope ps(c, NSG_PROF_SPLIT, 0.0);
  split_tf32_kernel<<<grid, 256, 0, c->stream>>>(src, rows, K, rs, ks, bs, rows_p, K_p, hi, lo, batch);
  count_launch(c);
  check_launch("split_tf32");
}

}  // namespace

bool gemm_split_tc(nsg_ctx* c, const GemmArgs& g) {
  if (c->precision != NSG_PREC_TF32X3) return false;
  if (g.dtype != NSG_F64) return false;
  if (g.opA == OP_C || g.opA == OP_R || g.opB == OP_C || g.opB == OP_R) return false;
  // small products stay on the FP64 path (tensor cores need full 128-row tiles to pay off)
  if (g.M < 64 || g.N < 64 || g.K < 32) return false;
  if (g.batch > 65535) return false;
  const int64_t Mp = (g.M + TM - 1) / TM * TM, Np = (g.N + BN - 1) / BN * BN, Kp = (g.K + BK - 1) / BK * BK;
  // A(r, k): op N -> A[r + k*lda]; op T -> A[k + r*lda]
  const int64_t ars = (g.opA == OP_N) ? 1 : g.lda, aks = (g.opA == OP_N) ? g.lda : 1;
  // B^T(n, k) = B(k, n): op N -> B[k + n*ldb]; op T -> B[n + k*ldb]
  const int64_t brs = (g.opB == OP_N) ? g.ldb : 1, bks = (g.opB == OP_N) ? 1 : g.ldb;
  const int64_t aB = g.strideA, bB = g.strideB;
  const int64_t ab = (aB == 0) ? 1 : g.batch, bb = (bB == 0) ? 1 : g.batch;
  if (g.batch > 1 && (ab == 1 || bb == 1)) return false;
  size_t szA = size_t(Mp) * Kp * ab, szB = size_t(Np) * Kp * bb;
  ScopedBuf sbuf(c, sizeof(float) * 2 * (szA + szB));
  float* Ah = (float*)sbuf.p;
  float* Al = Ah + szA;
  float* Bh = Al + szA;
  float* Bl = Bh + szB;
  split_operand(c, (const double*)g.A, g.M, g.K, ars, aks, aB, ab, Mp, Kp, Ah, Al);
  split_operand(c, (const double*)g.B, g.N, g.K, brs, bks, bB, bb, Np, Kp, Bh, Bl);
  CUtensorMap mAh = make_map(Ah, Mp, Kp, ab, TM), mAl = make_map(Al, Mp, Kp, ab, TM);
  CUtensorMap mBh = make_map(Bh, Np, Kp, bb, BN), mBl = make_map(Bl, Np, Kp, bb, BN);
  int* err = device_flag(c);  // checked once at the end of the public call
  ensure_smem_limit((const void*)tc_gemm_tf32x3_kernel, SMEM_BYTES);
  EpiParams ep{(double*)g.C, g.ldc, g.strideC, g.M, g.N, g.alpha_re, g.beta_re, err};
  dim3 grid(unsigned(Mp / TM), unsigned(Np / BN), unsigned(g.batch));
  {
  ProfScope ps(c, NSG_PROF_TC_GEMM, 2.0 * double(g.M) * double(g.N) * double(g.K) * double(g.batch));
  tc_gemm_tf32x3_kernel<<<grid, NTHREADS, SMEM_BYTES, c->stream>>>(mAh, mAl, mBh, mBl, int(Kp / BK), ep);
  }
  count_launch(c);
  check_launch("tc_gemm_tf32x3");
  return true;
}

}  // namespace nsg

// ---------------------------------------------------------------------------
// Allocation-free variant of the TF32x3 split-precision GEMM.
//
// Some callers must not allocate device memory behind their own allocator: a Julia
// program using CUDA.jl hands the device to CUDA.jl's memory pool, which has usually
// reserved most of HBM already, so a library cudaMalloc can fail or push the pool into
// out-of-memory; a host that runs this GEMM between operations of its own caching
// allocator (PyTorch, RMM) wants every byte accounted for by that allocator; and a
// latency-bound caller cannot afford the device-wide synchronisation cudaMalloc and
// cudaFree may imply.  For them the slice buffers and the error flag of this GEMM live
// in one statically sized device array that every GPU loading the library holds until
// the process exits.
// ---------------------------------------------------------------------------

namespace nsg {
namespace {

// 64 MiB of TF32 slices (hi and lo of op(A) and op(B), padded) plus a 256-byte header
// that holds the device-side error flag.
constexpr size_t kNoAllocSliceBytes = size_t(64) << 20;
constexpr size_t kNoAllocHeader = 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHeader + kNoAllocSliceBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};
int g_noalloc_sms[kMaxDevices] = {};

void noalloc_error(char* buf, int len, const std::string& msg) {
  if (buf && len > 0) {
    size_t n = std::min<size_t>(size_t(len - 1), msg.size());
    std::memcpy(buf, msg.data(), n);
    buf[n] = 0;
  }
}

}  // namespace

}  // namespace nsg

using namespace nsg;

extern "C" int nsg_gemm_tf32x3_noalloc(const double* A, int64_t lda, int transA, const double* B, int64_t ldb,
                                       int transB, double* C, int64_t ldc, int64_t M, int64_t N, int64_t K,
                                       double alpha, double beta, void* stream, char* errbuf, int errlen) {
  try {
    NSG_CHECK(A && B && C && M > 0 && N > 0 && K > 0, NSG_ERR_INVALID, "noalloc gemm: null operand or empty size");
    NSG_CHECK(lda >= (transA ? K : M) && ldb >= (transB ? N : K) && ldc >= M, NSG_ERR_INVALID,
              "noalloc gemm: leading dimension too small");
    // each extent alone below the scratch's element count, so the padded sizes and their
    // product below cannot wrap (at most 2 x 2^24 x 2^24 x 8 bytes)
    constexpr int64_t kMaxExtent = int64_t(kNoAllocSliceBytes / 8);
    NSG_CHECK(M <= kMaxExtent && N <= kMaxExtent && K <= kMaxExtent, NSG_ERR_UNSUPPORTED,
              "noalloc gemm: an extent exceeds " + std::to_string(kMaxExtent) +
                  ", beyond the static scratch maximum (use the allocating entry points)");
    const int64_t Mp = (M + TM - 1) / TM * TM, Np = (N + BN - 1) / BN * BN, Kp = (K + BK - 1) / BK * BK;
    const size_t need = sizeof(float) * 2 * size_t(Mp + Np) * size_t(Kp);
    NSG_CHECK(need <= kNoAllocSliceBytes, NSG_ERR_UNSUPPORTED,
              "noalloc gemm: operands need " + std::to_string(need) + " bytes of slice scratch, above the static " +
                  std::to_string(kNoAllocSliceBytes) + "-byte maximum (use the allocating entry points)");
    int dev = 0;
    NSG_CUDA(cudaGetDevice(&dev));
    NSG_CHECK(dev >= 0 && dev < kMaxDevices, NSG_ERR_UNSUPPORTED, "noalloc gemm: device index too large");
    unsigned char* base = nullptr;
    int sms = 0;
    {
      // one-time set-up per device, with that device current: resolve the static array's
      // device address and opt the kernel into its shared-memory size
      std::lock_guard<std::mutex> lk(g_noalloc_mu);
      if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        NSG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        NSG_CUDA(cudaFuncSetAttribute(tc_gemm_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BYTES));
        NSG_CUDA(cudaDeviceGetAttribute(&g_noalloc_sms[dev], cudaDevAttrMultiProcessorCount, dev));
        g_noalloc_ptr[dev] = (unsigned char*)p;
      }
      base = g_noalloc_ptr[dev];
      sms = g_noalloc_sms[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    int* err = (int*)base;
    float* Ah = (float*)(base + kNoAllocHeader);
    float* Al = Ah + size_t(Mp) * Kp;
    float* Bh = Al + size_t(Mp) * Kp;
    float* Bl = Bh + size_t(Np) * Kp;
    // the flag keeps the previous call's value: clear it before this call's kernels
    NSG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    const int64_t ars = transA ? lda : 1, aks = transA ? 1 : lda;
    const int64_t brs = transB ? 1 : ldb, bks = transB ? ldb : 1;
    auto split = [&](const double* src, int64_t rows, int64_t rs, int64_t ks, int64_t rows_p, float* hi, float* lo) {
      int64_t ntiles = ((rows_p + 31) / 32) * (Kp / 32);
      int grid = int(std::min<int64_t>(ntiles, (int64_t)sms * 16));
      split_tf32_kernel<<<grid, 256, 0, st>>>(src, rows, K, rs, ks, 0, rows_p, Kp, hi, lo, 1);
      check_launch("noalloc split_tf32");
    };
    split(A, M, ars, aks, Mp, Ah, Al);
    split(B, N, brs, bks, Np, Bh, Bl);
    CUtensorMap mAh = make_map(Ah, Mp, Kp, 1, TM), mAl = make_map(Al, Mp, Kp, 1, TM);
    CUtensorMap mBh = make_map(Bh, Np, Kp, 1, BN), mBl = make_map(Bl, Np, Kp, 1, BN);
    EpiParams ep{C, ldc, 0, M, N, alpha, beta, err};
    dim3 grid(unsigned(Mp / TM), unsigned(Np / BN), 1u);
    tc_gemm_tf32x3_kernel<<<grid, NTHREADS, SMEM_BYTES, st>>>(mAh, mAl, mBh, mBl, int(Kp / BK), ep);
    check_launch("noalloc tc_gemm_tf32x3");
    int herr = 0;
    NSG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSG_CUDA(cudaStreamSynchronize(st));
    NSG_CHECK(herr == 0, NSG_ERR_TIMEOUT, "noalloc gemm: a bounded mbarrier wait timed out");
  } catch (const Error& e) {
    noalloc_error(errbuf, errlen, e.what());
    return e.code;
  } catch (const std::exception& e) {
    noalloc_error(errbuf, errlen, e.what());
    return NSG_ERR_INVALID;
  }
  noalloc_error(errbuf, errlen, "");
  return NSG_OK;
}
