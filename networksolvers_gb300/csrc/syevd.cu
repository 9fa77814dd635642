// Dense Hermitian eigensolver for the truncated factorizations:
//   1. Householder reduction to a real symmetric tridiagonal T: one thread-block
//      cluster holding the matrix in distributed shared memory (orders up to the tuning
//      table's limit), else one cooperative kernel over all SMs with one grid barrier
//      per column (the matrix stays L2-resident),
//   2. Cuppen divide and conquer on T: implicit-QL leaves (8 rows by default), rank-one
//      merges with deflation (small z / close poles), every merge of a tree level in one
//      launch per step, secular roots by the two-pole rational model inside a bracket
//      with the origin at the nearer pole (one warp per root), Gu-Eisenstat recomputed z
//      for orthogonal vectors, merged by one batched product per level,
//   3. back-transformation of the kept eigenvectors with the Householder reflectors
//      in blocks of 64 (compact WY, three GEMMs per block; every block's T factor is
//      formed up front in one launch).
// The merge GEMMs and the two large back-transformation GEMMs use the FP64-level
// products (eight-slice Ozaki form in the split precision); the reflector Gram matrix
// V^H V and T W stay on the FP64 cores (six-slice products there alone cost 1e-11 of
// orthogonality).
// Every wait in these kernels is bounded: the grid barrier gives up after ~2^26
// polls, raises an error flag and the host reports NSG_ERR_TIMEOUT.
#include "nsg_internal.h"
#include "tuning_table.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>

namespace nsg {


static void raise_smem_limit(const void* fn, int bytes) { ensure_smem_limit(fn, bytes); }

namespace {

constexpr int kLeaf = 32;
constexpr int kTriUnits = 1024;  // pass work units per CTA and step (columns x row blocks)

__device__ __forceinline__ double cre(double v) { return v; }
__device__ __forceinline__ double cre(double2 v) { return v.x; }
__device__ __forceinline__ double cabs2(double v) { return v * v; }
__device__ __forceinline__ double cabs2(double2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ double cconj(double v) { return v; }
__device__ __forceinline__ double2 cconj(double2 v) { return make_double2(v.x, -v.y); }
__device__ __forceinline__ double cmulv(double a, double b) { return a * b; }
__device__ __forceinline__ double2 cmulv(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double cscale(double a, double s) { return a * s; }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double cadd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double csub(double a, double b) { return a - b; }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
template <typename T>
__device__ __forceinline__ T czero();
template <>
__device__ __forceinline__ double czero<double>() { return 0.0; }
template <>
__device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <typename T>
__device__ __forceinline__ T cone();
template <>
__device__ __forceinline__ double cone<double>() { return 1.0; }
template <>
__device__ __forceinline__ double2 cone<double2>() { return make_double2(1.0, 0.0); }
__device__ __forceinline__ double cdiv(double a, double b) { return a / b; }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  double den = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

// v - a b - c d and acc + conj(a) b as chains of fused multiply-adds (two FP64
// operations per real element: the FP64 pipe bounds the tridiagonalisation)
__device__ __forceinline__ double fnms2(double v, double a, double b, double c, double d) {
  return fma(-c, d, fma(-a, b, v));
}
__device__ __forceinline__ double2 fnms2(double2 v, double2 a, double2 b, double2 c, double2 d) {
  double re = fma(c.y, d.y, fma(-c.x, d.x, fma(a.y, b.y, fma(-a.x, b.x, v.x))));
  double im = fma(-c.y, d.x, fma(-c.x, d.y, fma(-a.y, b.x, fma(-a.x, b.y, v.y))));
  return make_double2(re, im);
}
__device__ __forceinline__ double fcma(double acc, double a, double b) { return fma(a, b, acc); }
__device__ __forceinline__ double2 fcma(double2 acc, double2 a, double2 b) {
  return make_double2(fma(a.y, b.y, fma(a.x, b.x, acc.x)), fma(-a.y, b.x, fma(a.x, b.y, acc.y)));
}

// Grid barrier state of the tridiagonalisation (cooperative launch guarantees
// co-residency): a monotonic arrival counter (every CTA knows how many arrivals close
// each step, so nothing is reset between steps) and an error flag set by a wait that
// gave up.
struct Barrier {
  unsigned int count;
  int err;
};

// Householder scalars of a pivot column whose first entry below the diagonal is alpha
// and whose further entries have squared norm xnorm2: beta = -sign(Re alpha) times the
// column's norm, tau = (beta - alpha) / beta and the scale 1 / (alpha - beta) that turns
// the column into the reflector v (v[0] = 1).  A zero tail under a real alpha needs no
// reflection (tau = 0, beta = alpha).
template <typename T>
__device__ __forceinline__ void hh_scalars(T alpha, double xnorm2, T& tk, T& scale, double& beta, bool& active) {
  const double ar = cre(alpha);
  double ai = 0.0;
  if constexpr (sizeof(T) == 16) ai = ((double2&)alpha).y;
  tk = czero<T>();
  scale = czero<T>();
  beta = ar;
  active = !(xnorm2 == 0.0 && ai == 0.0);
  if (active) {
    const double nrm = sqrt(ar * ar + ai * ai + xnorm2);
    beta = ar >= 0 ? -nrm : nrm;
    if constexpr (sizeof(T) == 16) {
      double2 t2 = make_double2((beta - ar) / beta, -ai / beta);
      tk = *(T*)&t2;
      double2 inv = cdiv(make_double2(1.0, 0.0), make_double2(ar - beta, ai));
      scale = *(T*)&inv;
    } else {
      double t1 = (beta - ar) / beta, s1 = 1.0 / (ar - beta);
      tk = *(T*)&t1;
      scale = *(T*)&s1;
    }
  }
}

// hh_scalars by one warp, its quotients spread over lanes (each lane runs the same
// division on its own operands: one division sequence instead of two, or four for
// complex data); lane 0 stores the results.  Same values as hh_scalars.
template <typename T>
__device__ __forceinline__ void hh_scalars_warp(T alpha, double xnorm2, int lane, T& tk, T& scale, double& beta,
                                                bool& active) {
  // lane 0's operands for every lane: the branch below holds full-warp shuffles, so it
  // must be uniform over the warp whatever the caller's lanes hold
  xnorm2 = __shfl_sync(0xffffffffu, xnorm2, 0);
  const double ar = __shfl_sync(0xffffffffu, cre(alpha), 0);
  double ai = 0.0;
  if constexpr (sizeof(T) == 16) ai = __shfl_sync(0xffffffffu, ((double2&)alpha).y, 0);
  const bool act = !(xnorm2 == 0.0 && ai == 0.0);
  double bt = ar;
  T t = czero<T>(), s = czero<T>();
  if (act) {
    const double nrm = sqrt(ar * ar + ai * ai + xnorm2);
    bt = ar >= 0 ? -nrm : nrm;
    if constexpr (sizeof(T) == 16) {
      // tau = ((beta - ar) / beta, -ai / beta), scale = 1 / (ar - beta + i ai)
      const double zx = ar - bt, zy = ai;
      const double den = zx * zx + zy * zy;
      const double num = lane == 0 ? bt - ar : lane == 1 ? -ai : lane == 2 ? zx : -zy;
      const double dv = lane < 2 ? bt : den;
      const double qv = num / dv;
      const double q0 = __shfl_sync(0xffffffffu, qv, 0), q1 = __shfl_sync(0xffffffffu, qv, 1);
      const double q2 = __shfl_sync(0xffffffffu, qv, 2), q3 = __shfl_sync(0xffffffffu, qv, 3);
      double2 t2 = make_double2(q0, q1), s2 = make_double2(q2, q3);
      t = *(T*)&t2;
      s = *(T*)&s2;
    } else {
      const double qv = (lane == 0 ? bt - ar : 1.0) / (lane == 0 ? bt : ar - bt);
      const double q0 = __shfl_sync(0xffffffffu, qv, 0), q1 = __shfl_sync(0xffffffffu, qv, 1);
      t = *(T*)&q0;
      s = *(T*)&q1;
    }
  }
  if (lane == 0) {
    tk = t;
    scale = s;
    beta = bt;
    active = act;
  }
}

// Householder tridiagonalisation of the Hermitian n x n matrix A (column-major, both
// triangles stored).  On exit d[k] = T_kk, e[k] = T_k,k+1 (real), tau[k], the reflector
// vectors v_k (v_k[k+1] = 1 implicit) below the subdiagonal of column k, and
// A[n-1, n-2] updated (its phase is handled by the caller for complex A).
// Step k: reflector from column k; x = tau A22 v; w = x - tau/2 (x^H v) v;
// A22 -= v w^H + w v^H.  The rank-2 update of step k-1 is applied lazily: every CTA
// rebuilds the updated pivot column itself, and one pass over the trailing block both
// applies the pending update and forms step k's x (one grid barrier per column).  CTAs
// retire as the trailing block shrinks (the barrier target follows the active count).
// A step is a chain of dependent L2 round trips, so the loads it needs are issued
// together: right after a barrier the next pivot column, x and the CTAs' partial sums,
// and at the top of a step the first tile of its pass.
template <typename T, int NT>
__global__ void __launch_bounds__(NT)
    tridiag_kernel(T* __restrict__ A, int n, double* __restrict__ d, double* __restrict__ e, T* __restrict__ tau,
                   T* __restrict__ xbuf, T* __restrict__ partial, Barrier* bar, int per_thread) {
  extern __shared__ unsigned char smem_raw[];
  T* vprev = (T*)smem_raw;  // pending update (relative to rows >= k)
  T* wprev = vprev + n;
  T* vcur = wprev + n;      // current reflector (relative to rows >= k+1)
  __shared__ T red[NT / 32];
  __shared__ double2 wsum[NT / 32];
  __shared__ T part_s[kTriUnits];  // per-unit partial dot products of the pass
  __shared__ int s_ok;
  __shared__ T a0_s[kTriUnits];    // first entry (row k+1) of each own column after the update
  __shared__ T s_tk, s_scale, s_alpha2;  // the step's scalars, formed by one warp
  __shared__ double s_beta;
  __shared__ bool s_active;
  constexpr int nt = NT, nwarps = NT / 32;
  static_assert(nwarps >= 2 && (nwarps & (nwarps - 1)) == 0, "warp 0 plus pass warps, a power of two");
  constexpr bool cplx = sizeof(T) == 16;   // real data: the imaginary halves are never formed
  constexpr int P = (cplx ? 1024 : 2048) / NT;  // pivot-column and x entries per thread held in registers
  constexpr int PQ = 8;                      // CTA partial sums per lane held in registers
  constexpr int U = sizeof(T) == 8 ? 16 : 8, RB = 32 * U;
  const int tid = threadIdx.x, b = blockIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  bool has_prev = false;
  unsigned int target = 0;  // arrivals on the barrier counter that close the current step
  // step 0's pivot column as stored: rows 1 + tid + j nt, and the diagonal
  T raw[P];
  T rawd = czero<T>();
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int r = tid + j * nt;
    raw[j] = r < n - 1 ? __ldcg(A + 1 + r) : czero<T>();
  }
  if (b == 0 && tid == 0) rawd = __ldcg(A);
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;  // trailing size (rows k+1..n-1)
    // (32-bit index arithmetic: the order is at most ~8.5k, so m^2 and m x CTAs fit)
    int nact = (m * m + nt * per_thread - 1) / (nt * per_thread);
    nact = max(1, min(nact, (int)gridDim.x));
    if (b >= nact) return;
    // x and the partial sums are double-buffered by step parity: a CTA that runs ahead
    // writes the other buffer while a slower one still reads this step's values (the
    // barrier keeps every CTA within one step of the others)
    T* xb = xbuf + (size_t)(k & 1) * n;
    double2* pb = (double2*)partial + (size_t)(k & 1) * gridDim.x;
    // the CTA's columns [j0, j1) of the trailing block, in work units of one column x RB
    // rows dealt round-robin to the pass warps (every warp but warp 0, which forms the
    // step's scalars meanwhile: their chain of dependent FP64 operations would otherwise
    // delay warp 0's units); the block is final since the last barrier, so each pass
    // warp's first unit is requested before the pivot column is reduced
    const int j0 = m * b / nact, j1 = m * (b + 1) / nact;
    const int ncol = j1 - j0, nrb = (m + RB - 1) / RB, nunits = ncol * nrb;
    constexpr int PW = nwarps - 1;
    const int pw = warp - 1;
    T cur[U], nxt[U];
    auto load_unit = [&](int u, T* dst) {
      const int q = u / nrb, rb = u - q * nrb;
      const T* cj = A + (size_t)(k + 1 + j0 + q) * n + (k + 1);
#pragma unroll
      for (int t = 0; t < U; ++t) {
        const int r = rb * RB + 32 * t + lane;
        dst[t] = r < m ? __ldcg(cj + r) : czero<T>();
      }
    };
    if (warp > 0 && pw < nunits) load_unit(pw, cur);
    // 1. pivot column k with the pending update applied (rows k..n-1), reflector
    const T* colk = A + (size_t)k * n;
    const T wp0 = has_prev ? cconj(wprev[0]) : czero<T>();
    const T vp0 = has_prev ? cconj(vprev[0]) : czero<T>();
    T dk = czero<T>();
    if (b == 0 && tid == 0) dk = has_prev ? fnms2(rawd, vprev[0], wp0, wprev[0], vp0) : rawd;
    double ss = 0.0, ss1 = 0.0;  // two chains of dependent FP64 additions
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int r = tid + j * nt;
      if (r < m) {
        T a = raw[j];
        if (has_prev) a = fnms2(a, vprev[r + 1], wp0, wprev[r + 1], vp0);
        vcur[r] = a;
        if (r > 0) {
          if (j & 1)
            ss1 += cabs2(a);
          else
            ss += cabs2(a);
        }
      }
    }
    ss += ss1;
    for (int r = tid + P * nt; r < m; r += nt) {  // orders above P nt + 1: loaded here
      T a = __ldcg(colk + k + 1 + r);
      if (has_prev) a = fnms2(a, vprev[r + 1], wp0, wprev[r + 1], vp0);
      vcur[r] = a;
      ss += cabs2(a);
    }
    // the squared norm: warp sums, then warp 0 adds them in warp order and forms the
    // reflector's scalars while the other warps start the pass (a warp-wide FP64
    // instruction holds a sub-partition's FP64 pipe for ~64 cycles on this GPU: the
    // scalar chain of square root and divides runs once per CTA, beside the pass).  The
    // pass needs no scalar: with v_0 = 1 and v_i = scale a_i (i > 0), where
    // alpha - beta = 1 / scale, A^H v = scale (A^H a - beta conj(A_0,:)); it forms A^H a
    // with the column as it is and keeps each column's first entry (a0_s).
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, o);
    if (lane == 0) ((double*)red)[warp] = ss;
    __syncthreads();  // publishes vcur (the column a, unscaled) and the warp sums
    if (warp == 0) {
      // a tree over the warps' sums (lane 0 ends with the total; hh_scalars_warp takes
      // lane 0's operands for every lane)
      double xnorm2 = lane < nwarps ? ((double*)red)[lane] : 0.0;
      for (int o = nwarps / 2; o > 0; o >>= 1) xnorm2 += __shfl_xor_sync(0xffffffffu, xnorm2, o);
      hh_scalars_warp(vcur[0], xnorm2, lane, s_tk, s_scale, s_beta, s_active);
      if (b == 0 && lane == 0) {
        d[k] = cre(dk);
        e[k] = s_active ? s_beta : cre(vcur[0]);
        tau[k] = s_tk;
      }
    }
    // 2. the pass: pending update, then the dot products of the columns with a.  A warp
    //    loads its next unit before it updates and stores the current one (units are
    //    disjoint).  The trailing block is rewritten by other CTAs between steps: every
    //    access bypasses L1.
    T tk, scale;
    bool active;
    {
      for (int u = warp > 0 ? pw : nunits; u < nunits; u += PW) {
        if (u + PW < nunits) load_unit(u + PW, nxt);
        const int q = u / nrb, rb = u - q * nrb, jj = j0 + q;
        T* cj = A + (size_t)(k + 1 + jj) * n + (k + 1);
        const T wj = has_prev ? cconj(wprev[jj + 1]) : czero<T>();
        const T vj = has_prev ? cconj(vprev[jj + 1]) : czero<T>();
        T acc = czero<T>(), acc1 = czero<T>();
#pragma unroll
        for (int t = 0; t < U; ++t) {
          const int r = rb * RB + 32 * t + lane;
          if (r < m) {
            T val = cur[t];
            if (has_prev) {
              val = fnms2(val, vprev[r + 1], wj, wprev[r + 1], vj);
              __stcg(cj + r, val);
            }
            if (t == 0 && r == 0) a0_s[q] = val;
            if (t & 1)
              acc1 = fcma(acc1, val, vcur[r]);
            else
              acc = fcma(acc, val, vcur[r]);
          }
        }
        acc = cadd(acc, acc1);
        for (int o = 16; o > 0; o >>= 1) {
          if constexpr (sizeof(T) == 8) {
            acc += __shfl_down_sync(0xffffffffu, acc, o);
          } else {
            double2 t2;
            t2.x = __shfl_down_sync(0xffffffffu, ((double2&)acc).x, o);
            t2.y = __shfl_down_sync(0xffffffffu, ((double2&)acc).y, o);
            acc = cadd(acc, *(T*)&t2);
          }
        }
        if (lane == 0) part_s[u] = acc;
#pragma unroll
        for (int t = 0; t < U; ++t) cur[t] = nxt[t];
      }
      __syncthreads();  // publishes the partial sums, a0_s and the scalars
      tk = s_tk;
      scale = s_scale;
      active = s_active;
      const double beta = s_beta;
      const T ts = cmulv(tk, scale);
      // column sums in a fixed order, x, and this CTA's share of x^H v (a warp whose
      // threads own no column contributes nothing and skips its reduction)
      const int cwarps = (ncol + 31) / 32;
      if (warp < cwarps) {
        double2 pacc = make_double2(0.0, 0.0);
        for (int q = tid; q < ncol; q += nt) {
          T sum = czero<T>();
          for (int rb = 0; rb < nrb; ++rb) sum = cadd(sum, part_s[q * nrb + rb]);
          const T xi = cmulv(ts, csub(sum, cscale(cconj(a0_s[q]), beta)));
          __stcg(xb + j0 + q, xi);
          const T vq = (j0 + q == 0) ? cone<T>() : cmulv(scale, vcur[j0 + q]);
          const T p = cmulv(cconj(xi), vq);
          if constexpr (!cplx) {
            pacc.x += (double&)p;
          } else {
            pacc.x += ((double2&)p).x;
            pacc.y += ((double2&)p).y;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          pacc.x += __shfl_down_sync(0xffffffffu, pacc.x, o);
          if constexpr (cplx) pacc.y += __shfl_down_sync(0xffffffffu, pacc.y, o);
        }
        if (lane == 0) wsum[warp] = pacc;
      }
      __syncthreads();
      // the reflector v itself (v_0 = 1) for the update, its storage and the next step
      for (int r = tid; r < m; r += nt) vcur[r] = (r == 0) ? cone<T>() : cmulv(vcur[r], scale);
      if (tid == 0) {
        double2 sacc = cwarps > 0 ? wsum[0] : make_double2(0.0, 0.0);
        for (int w = 1; w < cwarps; ++w) {
          sacc.x += wsum[w].x;
          if constexpr (cplx) sacc.y += wsum[w].y;
        }
        __stcg(pb + b, sacc);
      }
    }
    // 3. barrier among the active CTAs: every CTA active now was active in every earlier
    //    step (the active count never grows), so all of them agree on the target
    target += unsigned(nact);
    __syncthreads();
    if (tid == 0) {
      // arrival with release semantics (the block barrier above orders every thread's
      // stores of this step before it), polling with acquire semantics (the peers' stores
      // are visible after it, and the block barrier below passes that on): the same
      // ordering as full fences on both sides, without their cost
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&bar->count), "r"(1u) : "memory");
      long long polls = 0;
      for (;;) {
        unsigned int cnt;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cnt) : "l"(&bar->count) : "memory");
        if (int(cnt - target) >= 0) break;
        if (++polls > (1ll << 26) || *(volatile int*)&bar->err) {
          atomicExch(&bar->err, 1);
          break;
        }
        __nanosleep(20);
      }
      s_ok = (*(volatile int*)&bar->err) == 0;
    }
    __syncthreads();
    if (!s_ok) return;
    // 4. requested together: x, the CTAs' partials of x^H v, and the next pivot column
    //    (column k+1: rows k+2.. and its diagonal) as the pass above stored it
    T xr[P];
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int r = tid + j * nt;
      xr[j] = r < m ? __ldcg(xb + r) : czero<T>();
    }
    double2 pq[PQ];
    if (warp == 0) {
#pragma unroll
      for (int j = 0; j < PQ; ++j) {
        const int q = lane + 32 * j;
        pq[j] = q < nact ? __ldcg(pb + q) : make_double2(0.0, 0.0);
      }
    }
    {
      const T* coln = A + (size_t)(k + 1) * n + (k + 2);
#pragma unroll
      for (int j = 0; j < P; ++j) {
        const int r = tid + j * nt;
        raw[j] = r < m - 1 ? __ldcg(coln + r) : czero<T>();
      }
      if (b == 0 && tid == 0) rawd = __ldcg(A + (size_t)(k + 1) * n + (k + 1));
    }
    for (int r = tid + P * nt; r < m; r += nt) wprev[r] = __ldcg(xb + r);
    // warp 0 sums the CTAs' partials (lane-strided in ascending order, then a butterfly:
    // the same value in every CTA) and forms alpha2 for the CTA
    if (warp == 0) {
      // a tree over the lane's partials, then over the lanes
#pragma unroll
      for (int h = PQ / 2; h > 0; h >>= 1)
#pragma unroll
        for (int j = 0; j < h; ++j) {
          pq[j].x += pq[j + h].x;
          if constexpr (cplx) pq[j].y += pq[j + h].y;
        }
      double2 xv = pq[0];
      for (int q = lane + 32 * PQ; q < nact; q += 32) {
        const double2 t = __ldcg(pb + q);
        xv.x += t.x;
        if constexpr (cplx) xv.y += t.y;
      }
      for (int o = 16; o > 0; o >>= 1) {
        xv.x += __shfl_xor_sync(0xffffffffu, xv.x, o);
        if constexpr (cplx) xv.y += __shfl_xor_sync(0xffffffffu, xv.y, o);
      }
      if (lane == 0) {
        T xvT;
        if constexpr (sizeof(T) == 8) {
          double t1 = xv.x;
          xvT = *(T*)&t1;
        } else {
          xvT = *(T*)&xv;
        }
        s_alpha2 = cscale(cmulv(tk, xvT), -0.5);
      }
    }
    __syncthreads();
    const T alpha2 = s_alpha2;
    // reflector storage below the subdiagonal of column k: every CTA has read column k
    // before the barrier, and it is not read again
    if (b == 0)
      for (int r = tid + 1; r < m; r += nt) A[(size_t)k * n + (k + 1 + r)] = vcur[r];
    // 5. w = x + alpha2 v becomes the pending update (relative to rows >= k+1); a thread
    //    rewrites only the entries it holds
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int r = tid + j * nt;
      if (r < m) {
        vprev[r] = vcur[r];
        wprev[r] = active ? cadd(xr[j], cmulv(alpha2, vcur[r])) : czero<T>();
      }
    }
    for (int r = tid + P * nt; r < m; r += nt) {
      vprev[r] = vcur[r];
      wprev[r] = active ? cadd(wprev[r], cmulv(alpha2, vcur[r])) : czero<T>();
    }
    has_prev = active;
    __syncthreads();
  }
  if (b == 0 && tid == 0) {
    // last 2 x 2 block with the pending update of step n-3 (relative to rows >= n-2)
    auto upd = [&](int i, int j) -> T {
      T a = __ldcg(A + i + (size_t)j * n);
      if (has_prev && n >= 3)
        a = csub(a, cadd(cmulv(vprev[i - (n - 2)], cconj(wprev[j - (n - 2)])),
                         cmulv(wprev[i - (n - 2)], cconj(vprev[j - (n - 2)]))));
      return a;
    };
    if (n >= 2) {
      T a11 = upd(n - 2, n - 2), a21 = upd(n - 1, n - 2), a22 = upd(n - 1, n - 1);
      d[n - 2] = cre(a11);
      e[n - 2] = cre(a21);
      d[n - 1] = cre(a22);
      A[(n - 1) + (size_t)(n - 2) * n] = a21;
    } else {
      d[0] = cre(A[0]);
    }
  }
}

// Householder tridiagonalisation of a Hermitian matrix of moderate order (n <= ~640) by
// one thread-block cluster: the matrix is held in the cluster's distributed shared
// memory (column j in CTA j mod C, C <= 16), so a step's data never leaves the SMs and
// its synchronisation is the hardware cluster barrier instead of a grid barrier over
// global memory.  Same reflectors, tau, d and e as tridiag_kernel (the back-
// transformation reads v_k below the subdiagonal of A's column k).
// Step k: every CTA reads the pivot column from its owner (DSMEM), forms the reflector
// (identically in every CTA: same data, same reduction order); each CTA forms
// x_j = tau A22[:, j]^H v for its own columns; barrier; every CTA gathers x, forms
// w = x - tau/2 (x^H v) v and applies A22 -= v w^H + w v^H to its own columns; barrier.
constexpr int kClusterTriThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kClusterTriThreads)
    tridiag_cluster_kernel(T* __restrict__ A, int n, double* __restrict__ d, double* __restrict__ e,
                           T* __restrict__ tau) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = int(cluster.num_blocks());
  const int rank = int(cluster.block_rank());
  const int ncol = (n - rank + C - 1) / C;  // columns j = rank + C q, q < ncol
  const int ncmax = (n + C - 1) / C;        // the layout is the same in every CTA (remote
                                            // reads address a peer's arrays by this offset)
  extern __shared__ __align__(16) unsigned char ct_smem[];
  T* cols = (T*)ct_smem;               // own columns, n rows each
  T* vcur = cols + (size_t)ncmax * n;  // reflector (rows k+1..n-1 at offsets 0..m-1)
  T* xloc = vcur + n;                  // x_j of own columns (by global column index)
  T* xall = xloc + n;                  // gathered x (rows k+1.. at offsets 0..)
  T* wv = xall + n;                    // w
  __shared__ T red[kClusterTriThreads / 32];
  __shared__ double redd[kClusterTriThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = kClusterTriThreads / 32;
  static_assert(NW >= 2 && (NW & (NW - 1)) == 0, "warp 0 plus dot-product warps, a power of two");
  for (int q = 0; q < ncol; ++q) {
    const T* src = A + (size_t)(rank + C * q) * n;
    for (int r = tid; r < n; r += blockDim.x) cols[(size_t)q * n + r] = src[r];
  }
  cluster.sync();
  // block sums end in one warp (the warps' sums added in warp order), which also forms
  // the step's scalars: on this GPU a warp-wide FP64 instruction holds a sub-partition's
  // FP64 pipe for ~64 cycles, so a scalar chain repeated by every warp would take the
  // CTA's FP64 issue for a step of its own
  __shared__ T s_tk, s_scl, s_alpha2;
  __shared__ double s_beta;
  __shared__ bool s_active;
  auto warp_sum_t = [&](T v) {
    for (int o = 16; o > 0; o >>= 1) {
      if constexpr (sizeof(T) == 8) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
      } else {
        double2 t2;
        t2.x = __shfl_xor_sync(0xffffffffu, ((double2&)v).x, o);
        t2.y = __shfl_xor_sync(0xffffffffu, ((double2&)v).y, o);
        v = cadd(v, *(T*)&t2);
      }
    }
    return v;
  };
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;
    const int owner = k % C;
    const T* pcol = cluster.map_shared_rank(cols, owner) + (size_t)(k / C) * n;
    // 1. the reflector from column k (rows k+1..n-1), in every CTA
    double ss = 0.0;
    for (int r = tid; r < m; r += blockDim.x) {
      const T a = pcol[k + 1 + r];
      vcur[r] = a;
      if (r > 0) ss += cabs2(a);
    }
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    if (lane == 0) redd[warp] = ss;
    __syncthreads();  // publishes vcur (the column a, unscaled) and the warp sums
    // warp 0 forms the reflector's scalars while the other warps form the dot products
    // S_j = sum_i conj(A_ij) a_i of the own trailing columns with the column as it is
    // (one warp per column): with v_0 = 1, v_i = scale a_i (i > 0) and
    // alpha - beta = 1 / scale, A^H v = scale (S - beta conj(A_0,:))
    if (warp == 0) {
      // a tree over the warps' sums (lane 0 ends with the total; hh_scalars_warp takes
      // lane 0's operands for every lane)
      double xnorm2 = lane < NW ? redd[lane] : 0.0;
      for (int o = NW / 2; o > 0; o >>= 1) xnorm2 += __shfl_xor_sync(0xffffffffu, xnorm2, o);
      hh_scalars_warp(vcur[0], xnorm2, lane, s_tk, s_scl, s_beta, s_active);
      if (rank == owner && lane == 0) {
        d[k] = cre(pcol[k]);
        e[k] = s_active ? s_beta : cre(vcur[0]);
        tau[k] = s_tk;
      }
    }
    // 2. x_j = tau sum_i conj(A_ij) v_i for the own trailing columns, one warp per column
    //    on the warps other than warp 0
    const int q0 = (k + 1 - rank + C - 1) / C;  // first own column index with j >= k+1
    for (int q = warp > 0 ? q0 + warp - 1 : ncol; q < ncol; q += NW - 1) {
      const int j = rank + C * q;
      const T* cj = cols + (size_t)q * n + (k + 1);
      T acc = czero<T>(), acc1 = czero<T>();
      int r = lane;
      for (; r + 32 < m; r += 64) {
        acc = fcma(acc, cj[r], vcur[r]);
        acc1 = fcma(acc1, cj[r + 32], vcur[r + 32]);
      }
      if (r < m) acc = fcma(acc, cj[r], vcur[r]);
      acc = cadd(acc, acc1);
      for (int o = 16; o > 0; o >>= 1) {
        if constexpr (sizeof(T) == 8) {
          acc += __shfl_xor_sync(0xffffffffu, acc, o);
        } else {
          double2 t2;
          t2.x = __shfl_xor_sync(0xffffffffu, ((double2&)acc).x, o);
          t2.y = __shfl_xor_sync(0xffffffffu, ((double2&)acc).y, o);
          acc = cadd(acc, *(T*)&t2);
        }
      }
      if (lane == 0) xloc[j] = acc;
    }
    __syncthreads();  // publishes the scalars and the dot products
    const T tk = s_tk, scl = s_scl;
    const bool active = s_active;
    {
      const double beta = s_beta;
      const T ts = cmulv(tk, scl);
      for (int q = q0 + tid; q < ncol; q += blockDim.x) {
        const int j = rank + C * q;
        xloc[j] = cmulv(ts, csub(xloc[j], cscale(cconj(cols[(size_t)q * n + (k + 1)]), beta)));
      }
    }
    for (int r = tid; r < m; r += blockDim.x) vcur[r] = (r == 0) ? cone<T>() : cmulv(vcur[r], scl);
    cluster.sync();  // publishes x to the peers and the scaled reflector within the CTA
    if (rank == owner) {
      T* gcol = A + (size_t)k * n + (k + 1);
      for (int r = tid + 1; r < m; r += blockDim.x) gcol[r] = vcur[r];
    }
    if (active) {
      // 3. gather x, x^H v, w = x - tau/2 (x^H v) v
      T pv = czero<T>();
      for (int r = tid; r < m; r += blockDim.x) {
        const int j = k + 1 + r;
        const T xj = cluster.map_shared_rank(xloc, j % C)[j];
        xall[r] = xj;
        pv = cadd(pv, cmulv(cconj(xj), vcur[r]));
      }
      pv = warp_sum_t(pv);
      if (lane == 0) red[warp] = pv;
      __syncthreads();
      if (warp == 0) {
        T xv = lane < NW ? red[lane] : czero<T>();  // a tree over the warps' sums (lane 0)
        for (int o = NW / 2; o > 0; o >>= 1) {
          if constexpr (sizeof(T) == 8) {
            xv += __shfl_xor_sync(0xffffffffu, xv, o);
          } else {
            double2 t2;
            t2.x = __shfl_xor_sync(0xffffffffu, ((double2&)xv).x, o);
            t2.y = __shfl_xor_sync(0xffffffffu, ((double2&)xv).y, o);
            xv = cadd(xv, *(T*)&t2);
          }
        }
        if (lane == 0) s_alpha2 = cscale(cmulv(tk, xv), -0.5);
      }
      __syncthreads();
      const T alpha2 = s_alpha2;
      for (int r = tid; r < m; r += blockDim.x) wv[r] = cadd(xall[r], cmulv(alpha2, vcur[r]));
      __syncthreads();
      // 4. A22 -= v w^H + w v^H on the own trailing columns
      for (int q = q0 + warp; q < ncol; q += NW) {
        const int jr = rank + C * q - (k + 1);
        T* cj = cols + (size_t)q * n + (k + 1);
        const T wj = cconj(wv[jr]), vj = cconj(vcur[jr]);
        for (int r = lane; r < m; r += 32) cj[r] = fnms2(cj[r], vcur[r], wj, wv[r], vj);
      }
    }
    cluster.sync();
  }
  // the last 2 x 2 block
  if (n >= 2) {
    const int o2 = (n - 2) % C, o1 = (n - 1) % C;
    if (rank == o2 && tid == 0) {
      const T* c2 = cols + (size_t)((n - 2) / C) * n;
      const T a11 = c2[n - 2], a21 = c2[n - 1];
      d[n - 2] = cre(a11);
      e[n - 2] = cre(a21);
      A[(n - 1) + (size_t)(n - 2) * n] = a21;
    }
    if (rank == o1 && tid == 0) d[n - 1] = cre(cols[(size_t)((n - 1) / C) * n + (n - 1)]);
  } else if (rank == 0 && tid == 0) {
    d[0] = cre(cols[0]);
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// For complex A the last subdiagonal element may be complex: handled on the host by a
// unitary diagonal scaling (phase folded into the back-transformation).

// ---------------------------------------------------------------------------
// divide and conquer
// ---------------------------------------------------------------------------

struct MergeDesc {
  int lo, mid, hi;
  double beta;
};


// Scatter leaf eigenpairs into Q (n x n, column-major) and w, sorted ascending.
// Leaves of the divide and conquer: the symmetric tridiagonal blocks (order <= 32) are
// diagonalised by the implicit QL method with Wilkinson shifts (Givens chase from the
// bottom of the unreduced block to its top), one warp per leaf.  Lane 0 runs each
// chase's scalar recurrence and records its rotations; then every lane applies them, in
// order, to its own row of the eigenvector matrix Z (columns = eigenvectors).  The
// eigenpairs are sorted ascending and written into the leaf's diagonal block of Q and w.
// A block that fails to converge in 60 chases per eigenvalue raises *err.
constexpr int kLeafWarps = 4;
__global__ void __launch_bounds__(32 * kLeafWarps)
    leaf_ql_kernel(const double* __restrict__ dsrc, const double* __restrict__ esrc, const int* leaf_lo,
                   const int* leaf_hi, int nleaf, double* Q, int n, double* w, int* err) {
  __shared__ double Zs[kLeafWarps][kLeaf][kLeaf + 1];
  __shared__ double ds_[kLeafWarps][kLeaf], es_[kLeafWarps][kLeaf], cs_[kLeafWarps][kLeaf],
      sn_[kLeafWarps][kLeaf];
  __shared__ int ord_[kLeafWarps][kLeaf];
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int L = blockIdx.x * kLeafWarps + wl;
  if (L >= nleaf) return;  // whole warps only
  const int lo = leaf_lo[L], s = leaf_hi[L] - lo;
  double(*Z)[kLeaf + 1] = Zs[wl];
  double* d = ds_[wl];
  double* e = es_[wl];
  for (int c = 0; c < kLeaf; ++c) Z[lane][c] = (lane == c) ? 1.0 : 0.0;
  if (lane < s) {
    d[lane] = dsrc[lo + lane];
    e[lane] = (lane + 1 < s) ? esrc[lo + lane] : 0.0;
  }
  __syncwarp();
  const double eps = 2.220446049250313e-16;
  bool failed = false;
  for (int l = 0; l < s && !failed; ++l) {
    for (int iter = 0;; ++iter) {
      int m = l;
      while (m < s - 1) {
        const double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) <= eps * dd) break;
        ++m;
      }
      if (m == l) break;
      if (iter == 60) {
        failed = true;
        break;
      }
      int lowest = l;  // rotations recorded for i = m-1 .. lowest
      if (lane == 0) {
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = sqrt(g * g + 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
        double sv = 1.0, cv = 1.0, p = 0.0;
        int i = m - 1;
        for (; i >= l; --i) {
          const double f = sv * e[i], b = cv * e[i];
          r = sqrt(f * f + g * g);
          e[i + 1] = r;
          if (r == 0.0) {  // the block splits: undo the pending shift and restart
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          const double ir = 1.0 / r;
          sv = f * ir;
          cv = g * ir;
          g = d[i + 1] - p;
          r = (d[i] - g) * sv + 2.0 * cv * b;
          p = sv * r;
          d[i + 1] = g + p;
          g = cv * r - b;
          cs_[wl][i] = cv;
          sn_[wl][i] = sv;
        }
        if (i < l) {
          d[l] -= p;
          e[l] = g;
          e[m] = 0.0;
        } else {
          lowest = i + 1;
        }
        ord_[wl][0] = lowest;
      }
      __syncwarp();
      lowest = ord_[wl][0];
      // each lane rotates its row of Z through the chase's rotations, in order
      for (int i = m - 1; i >= lowest; --i) {
        const double cv = cs_[wl][i], sv = sn_[wl][i];
        const double f = Z[lane][i + 1], zi = Z[lane][i];
        Z[lane][i + 1] = sv * zi + cv * f;
        Z[lane][i] = cv * zi - sv * f;
      }
      __syncwarp();
    }
  }
  if (failed && lane == 0) atomicExch(err, 1);
  // ascending order (insertion sort by lane 0), then the leaf's block of Q and w
  if (lane == 0) {
    int* o = ord_[wl];
    for (int a = 0; a < s; ++a) o[a] = a;
    for (int a = 1; a < s; ++a) {
      const int x = o[a];
      int b2 = a - 1;
      while (b2 >= 0 && d[o[b2]] > d[x]) {
        o[b2 + 1] = o[b2];
        --b2;
      }
      o[b2 + 1] = x;
    }
  }
  __syncwarp();
  if (lane < s) {
    for (int j = 0; j < s; ++j) Q[(size_t)(lo + j) * n + (lo + lane)] = Z[lane][ord_[wl][j]];
    w[lo + lane] = d[ord_[wl][lane]];
  }
}


// Merges of the divide and conquer, one tree level at a time: every kernel below
// handles all merges of a level in one launch (blockIdx.y or the warp index selects the
// merge), so a level costs a fixed handful of launches and one host read of the
// deflation counts, whatever the number of merges.
//
// Workspace (device arrays of length n; a merge uses the slice [lo, hi) of each):
//   Ds, zs     sorted (sign-flipped) poles and normalised z, 0 for deflated slots
//   perm       block-local column of sorted slot t
//   kind       1 = non-deflated, 0 = deflated
//   kinv       sorted slot of the q-th non-deflated pole
//   Dk, zk     the non-deflated poles and weights, compacted
//   lam, zh    secular roots and Gu-Eisenstat weights (first k entries)
//   srck, srci, wn   final ordering: source kind / index and eigenvalue of output column
//   rot_pq, rot_cs   deflation rotations (2 entries each per rotation, at 2 lo)
//   gscr       scratch of the serial steps for blocks above the shared-memory limit
// Per merge: rho, counts (k, nrot, flip).
struct DcWork {
  double *Ds, *zs, *Dk, *zk, *lam, *zh, *wn, *rot_cs, *gscr;
  int *perm, *kind, *kinv, *srck, *srci, *rot_pq;
  double* rho;
  int* counts;
};

constexpr int kSmemMerge = 4096;  // rows of a block whose serial steps run in shared memory

// Order-preserving integer key of a double (x < y exactly when key(x) < key(y); -0 and +0
// equal), so the merges compare with integer instructions rather than the FP64 pipe,
// and the exact negation -x by its sign bit.
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  if ((b & 0x7fffffffffffffffLL) == 0) return 0;
  return b < 0 ? (b ^ 0x7fffffffffffffffLL) : b;
}
__device__ __forceinline__ double neg_exact(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)(1ULL << 63));
}

// Exclusive prefix sum of v over the block's threads in thread order (sh: 32 ints);
// the block total goes to *tot.  Every thread of the block must call it.
__device__ int block_scan_excl(int v, int* sh, int* tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) sh[lane] = t;
  }
  __syncthreads();
  const int before = warp > 0 ? sh[warp - 1] : 0;
  *tot = sh[nw - 1];
  __syncthreads();
  return before + x - v;
}

// Number of indices i in [0, len) with key(i) < k (strict) or key(i) <= k, for keys
// ascending in i.
template <bool kStrict, typename F>
__device__ __forceinline__ int rank_in(F key, int len, long long k) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int md = (lo + hi) >> 1;
    const long long v = key(md);
    if (kStrict ? (v < k) : (v <= k))
      lo = md + 1;
    else
      hi = md;
  }
  return lo;
}

// Per merge (one CTA): gather the two halves' eigenvalues and the z vector (last row of
// block 1, first row of block 2), flip for rho < 0, merge the ascending halves, normalise
// z, deflate (small z_t; poles closer than tol rotated together), apply the deflation
// rotations to the block's columns of Q, and compact the non-deflated poles.
__global__ void dc_prep_kernel(const double* __restrict__ w, double* __restrict__ Q, int n,
                               const MergeDesc* __restrict__ md, DcWork W) {
  extern __shared__ double dp_smem[];
  const int mi = blockIdx.x;
  const MergeDesc M = md[mi];
  const int lo = M.lo, mid = M.mid, hi = M.hi, nb = hi - lo, n1 = mid - lo;
  const bool sm = nb <= kSmemMerge;
  double* ws = sm ? dp_smem : W.gscr + 2 * (size_t)lo;  // block eigenvalues by local index
  double* zr = ws + nb;                                  // z candidates by local index
  double* Dsm = sm ? zr + nb : W.Ds + lo;
  double* zsm = sm ? Dsm + nb : W.zs + lo;
  int* pm = sm ? (int*)(zsm + nb) : W.perm + lo;
  int* kd = sm ? pm + nb : W.kind + lo;
  __shared__ double red[32], redm[32];
  __shared__ int scan_sh[32], s_flag, s_nrot;
  for (int li = threadIdx.x; li < nb; li += blockDim.x) {
    ws[li] = w[lo + li];
    zr[li] = (li < n1) ? Q[(size_t)(lo + li) * n + (mid - 1)] : Q[(size_t)(lo + li) * n + mid];
  }
  if (threadIdx.x == 0) {
    s_flag = 0;
    s_nrot = 0;
  }
  __syncthreads();
  double rho = M.beta;
  const int flip = rho < 0;
  if (flip) rho = -rho;
  // merge of the two ascending halves (both traversed from their top when flipped, values
  // negated) into ascending poles; ties take the first half first.  An entry's slot is
  // its rank in its own half plus its rank in the other, by binary search on integer keys.
  const int n2 = nb - n1;
  auto srcA = [&](int a) { return flip ? (n1 - 1 - a) : a; };
  auto srcB = [&](int b2) { return flip ? (nb - 1 - b2) : (n1 + b2); };
  auto valA = [&](int a) { return flip ? neg_exact(ws[srcA(a)]) : ws[srcA(a)]; };
  auto valB = [&](int b2) { return flip ? neg_exact(ws[srcB(b2)]) : ws[srcB(b2)]; };
  auto keyA = [&](int a) { return order_key(valA(a)); };
  auto keyB = [&](int b2) { return order_key(valB(b2)); };
  for (int t = threadIdx.x; t < nb; t += blockDim.x)  // halves out of order: the serial merge
    if ((t > 0 && t < n1 && keyA(t) < keyA(t - 1)) || (t > n1 && keyB(t - n1) < keyB(t - n1 - 1))) s_flag = 1;
  __syncthreads();
  if (!s_flag) {
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      int pos, li;
      if (t < n1) {
        pos = t + rank_in<true>(keyB, n2, keyA(t));
        li = srcA(t);
      } else {
        pos = (t - n1) + rank_in<false>(keyA, n1, keyB(t - n1));
        li = srcB(t - n1);
      }
      pm[pos] = li;
      Dsm[pos] = flip ? neg_exact(ws[li]) : ws[li];
      zsm[pos] = zr[li];
    }
  } else if (threadIdx.x == 0) {
    int a = 0, b2 = 0;
    for (int t = 0; t < nb; ++t) {
      bool takeA;
      if (a >= n1)
        takeA = false;
      else if (b2 >= n2)
        takeA = true;
      else
        takeA = keyA(a) <= keyB(b2);
      const int li = takeA ? srcA(a) : srcB(b2);
      if (takeA)
        ++a;
      else
        ++b2;
      pm[t] = li;
      Dsm[t] = flip ? neg_exact(ws[li]) : ws[li];
      zsm[t] = zr[li];
    }
  }
  __syncthreads();
  // |z| and max |D| (fixed-order block reductions)
  double s2 = 0.0, dm = 0.0;
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    s2 += zsm[t] * zsm[t];
    dm = fmax(dm, fabs(Dsm[t]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0) {
    red[warp] = s2;
    redm[warp] = dm;
  }
  __syncthreads();
  double nz = 0.0, dmax = 0.0;
  for (int q = 0; q < nw; ++q) {
    nz += red[q];
    dmax = fmax(dmax, redm[q]);
  }
  nz = sqrt(nz);
  rho = rho * nz * nz;
  const double tol = 8.0 * 2.220446049250313e-16 * fmax(dmax, rho);
  // deflation of small weights (independent per pole), then of poles closer than tol:
  // the sorted poles' closest kept pair is consecutive among the kept ones, so a pass
  // that finds none proves that the serial rotation sweep would rotate nothing
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    const double z = zsm[t] / nz;
    const bool small = rho * fabs(z) <= tol;
    kd[t] = small ? 0 : 1;
    zsm[t] = small ? 0.0 : z;
  }
  if (threadIdx.x == 0) s_flag = 0;
  __syncthreads();
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    if (!kd[t]) continue;
    for (int u = t + 1; u < nb; ++u)
      if (kd[u]) {
        if (fabs(Dsm[u] - Dsm[t]) <= tol) s_flag = 1;
        break;
      }
  }
  __syncthreads();
  int* rpq = W.rot_pq + 2 * lo;
  double* rcs = W.rot_cs + 2 * lo;
  if (s_flag && threadIdx.x == 0) {
    int nrot = 0, prev = -1;
    for (int t = 0; t < nb; ++t) {
      if (!kd[t]) continue;
      if (prev >= 0 && fabs(Dsm[t] - Dsm[prev]) <= tol) {
        const double r = hypot(zsm[t], zsm[prev]);
        const double c = zsm[t] / r, sn = zsm[prev] / r;
        const double dp = Dsm[prev], dt = Dsm[t];
        Dsm[prev] = c * c * dp + sn * sn * dt;
        Dsm[t] = sn * sn * dp + c * c * dt;
        zsm[prev] = 0.0;
        zsm[t] = r;
        kd[prev] = 0;
        rpq[2 * nrot] = pm[prev];
        rpq[2 * nrot + 1] = pm[t];
        rcs[2 * nrot] = c;
        rcs[2 * nrot + 1] = sn;
        ++nrot;
      }
      prev = t;
    }
    s_nrot = nrot;
  }
  __syncthreads();
  // compaction of the non-deflated slots (block scan over contiguous chunks)
  {
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int c0 = min(nb, (int)threadIdx.x * per), c1 = min(nb, c0 + per);
    int cnt = 0;
    for (int t = c0; t < c1; ++t) cnt += kd[t];
    int k = 0;
    int off = block_scan_excl(cnt, scan_sh, &k);
    int* kinv = W.kinv + lo;
    double* Dk = W.Dk + lo;
    double* zk = W.zk + lo;
    for (int t = c0; t < c1; ++t)
      if (kd[t]) {
        kinv[off] = t;
        Dk[off] = Dsm[t];
        zk[off] = zsm[t];
        ++off;
      }
    if (threadIdx.x == 0) {
      W.rho[mi] = rho;
      W.counts[3 * mi] = k;
      W.counts[3 * mi + 1] = s_nrot;
      W.counts[3 * mi + 2] = flip;
    }
  }
  if (sm) {
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      W.Ds[lo + t] = Dsm[t];
      W.zs[lo + t] = zsm[t];
      W.perm[lo + t] = pm[t];
      W.kind[lo + t] = kd[t];
    }
  }
}

// The deflation rotations of every merge of a level, in order, on the block's columns of
// Q: one thread per row (blockIdx.y = merge), so a merge's rows are spread over many SMs
// and each thread's chain of dependent rotations is one row long.
__global__ void dc_rotate_kernel(double* __restrict__ Q, int n, const MergeDesc* __restrict__ md, DcWork W) {
  const int mi = blockIdx.y;
  const int nrot = W.counts[3 * mi + 1];
  if (nrot == 0) return;
  const int lo = md[mi].lo, nb = md[mi].hi - lo;
  const int* rpq = W.rot_pq + 2 * lo;
  const double* rcs = W.rot_cs + 2 * lo;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nb; r += gridDim.x * blockDim.x) {
    double* row = Q + (lo + r);
    for (int q = 0; q < nrot; ++q) {
      const size_t cp = (size_t)(lo + rpq[2 * q]) * n, ci = (size_t)(lo + rpq[2 * q + 1]) * n;
      const double c = rcs[2 * q], sn = rcs[2 * q + 1];
      const double xp = row[cp], xi = row[ci];
      row[cp] = c * xp - sn * xi;
      row[ci] = sn * xp + c * xi;
    }
  }
}

// Secular roots: one warp per (merge, root).  Root i of 1 + rho sum_j z_j^2 / (D_j - lambda)
// lies in (D_i, D_{i+1}) (the last one in (D_{k-1}, D_{k-1} + rho)); it is represented as
// origin + tau with the origin at the nearer pole, so D_j - lambda = (D_j - origin) - tau
// is exact enough for the Gu-Eisenstat vectors.  Iteration: the two-pole rational model
// of Bunch, Nielsen and Sorensen (psi for poles j <= i, phi for j > i, each matched in
// value and slope at tau), solved as a quadratic inside the bracket; bisection when the
// model step leaves the bracket.  Delta_m[i * k + j] = D_j - lambda_i (block of kmax^2).
__global__ void dc_secular_kernel(const MergeDesc* __restrict__ md, int nm, int kmax, DcWork W,
                                  double* __restrict__ Delta_all) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (gw >= (int64_t)nm * kmax) return;
  const int mi = int(gw / kmax), i = int(gw % kmax);
  const int k = W.counts[3 * mi];
  if (i >= k) return;
  const int lo = md[mi].lo;
  const double* Dk = W.Dk + lo;
  const double* zk = W.zk + lo;
  const double rho = W.rho[mi];
  double* Delta = Delta_all + (size_t)mi * kmax * kmax;
  const double eps = 2.220446049250313e-16;
  int org;
  double blo, bhi;
  if (i < k - 1) {
    const double gap = Dk[i + 1] - Dk[i];
    const double mid = 0.5 * gap;  // relative to D_i
    double f = 0.0;
    for (int j = lane; j < k; j += 32) f += rho * zk[j] * zk[j] / ((Dk[j] - Dk[i]) - mid);
    for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
    f += 1.0;
    if (f >= 0) {
      org = i;
      blo = 0.0;
      bhi = mid;
    } else {
      org = i + 1;
      blo = -mid;
      bhi = 0.0;
    }
  } else {
    org = k - 1;
    blo = 0.0;
    bhi = rho;
  }
  const double dorg = Dk[org];
  const double ddi = Dk[i] - dorg;
  const double ddi1 = (i < k - 1) ? Dk[i + 1] - dorg : 0.0;
  double tau = 0.5 * (blo + bhi);
  for (int it = 0; it < 100; ++it) {
    double psi = 0.0, dpsi = 0.0, phi = 0.0, dphi = 0.0, fa = 0.0;
    for (int j = lane; j < k; j += 32) {
      const double del = (Dk[j] - dorg) - tau;
      const double q = zk[j] / del;
      const double term = rho * zk[j] * q;
      const double dterm = rho * q * q;
      if (j <= i) {
        psi += term;
        dpsi += dterm;
      } else {
        phi += term;
        dphi += dterm;
      }
      fa += fabs(term);
    }
    for (int o = 16; o > 0; o >>= 1) {
      psi += __shfl_xor_sync(0xffffffffu, psi, o);
      dpsi += __shfl_xor_sync(0xffffffffu, dpsi, o);
      phi += __shfl_xor_sync(0xffffffffu, phi, o);
      dphi += __shfl_xor_sync(0xffffffffu, dphi, o);
      fa += __shfl_xor_sync(0xffffffffu, fa, o);
    }
    const double f = 1.0 + psi + phi;
    if (f > 0)
      bhi = tau;
    else
      blo = tau;
    if (fabs(f) <= 4.0 * eps * (k + 1.0) * (1.0 + fa)) break;
    if (bhi - blo <= 2.0 * eps * fmax(fabs(blo), fabs(bhi)) || bhi - blo < 1e-300) break;
    double tn;
    const double di = ddi - tau;
    const double b1 = dpsi * di * di, a1 = psi - b1 / di;
    if (i < k - 1) {
      const double di1 = ddi1 - tau;
      const double b2 = dphi * di1 * di1, a2 = phi - b2 / di1;
      const double C = 1.0 + a1 + a2;
      // C (ddi - x)(ddi1 - x) + b1 (ddi1 - x) + b2 (ddi - x) = 0
      const double qa = C, qb = -(C * (ddi + ddi1) + b1 + b2), qc = C * ddi * ddi1 + b1 * ddi1 + b2 * ddi;
      tn = NAN;
      if (qa != 0.0) {
        const double disc = qb * qb - 4.0 * qa * qc;
        if (disc >= 0.0) {
          const double sq = sqrt(disc);
          const double qq = -0.5 * (qb + copysign(sq, qb));
          const double r1 = qq / qa, r2 = (qq != 0.0) ? qc / qq : NAN;
          if (r1 > blo && r1 < bhi)
            tn = r1;
          else if (r2 > blo && r2 < bhi)
            tn = r2;
        }
      } else if (qb != 0.0) {
        tn = -qc / qb;
      }
    } else {
      // 1 + phi_const + a1 + b1/(ddi - x) = 0 with phi == 0
      const double C = 1.0 + a1 + phi;
      tn = (C != 0.0) ? ddi + b1 / C : NAN;
    }
    if (!(tn > blo && tn < bhi)) tn = 0.5 * (blo + bhi);
    if (tn == tau) break;
    tau = tn;
  }
  if (lane == 0) W.lam[lo + i] = dorg + tau;
  for (int j = lane; j < k; j += 32) Delta[(size_t)i * k + j] = (Dk[j] - dorg) - tau;
}

// Gu-Eisenstat: zhat_j^2 = (lam_j - D_j)/rho * prod_{i != j} (lam_i - D_j)/(D_i - D_j);
// one warp per (merge, j).
__global__ void dc_gu_eisenstat_kernel(const MergeDesc* __restrict__ md, int nm, int kmax, DcWork W,
                                       const double* __restrict__ Delta_all) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (gw >= (int64_t)nm * kmax) return;
  const int mi = int(gw / kmax), j = int(gw % kmax);
  const int k = W.counts[3 * mi];
  if (j >= k) return;
  const int lo = md[mi].lo;
  const double* Dk = W.Dk + lo;
  const double* Delta = Delta_all + (size_t)mi * kmax * kmax;
  double p = 1.0;
  for (int i = lane; i < k; i += 32)
    if (i != j) p *= (-Delta[(size_t)i * k + j]) / (Dk[i] - Dk[j]);
  for (int o = 16; o > 0; o >>= 1) p *= __shfl_xor_sync(0xffffffffu, p, o);
  p *= -Delta[(size_t)j * k + j] / W.rho[mi];
  if (lane == 0) W.zh[lo + j] = copysign(sqrt(fmax(p, 0.0)), W.zk[lo + j]);
}

// S^T of each merge (kmax x kmax, column-major, zero outside its k x k block: column i =
// normalised eigenvector of root i); one warp per (merge, column).
__global__ void dc_vectors_kernel(const MergeDesc* __restrict__ md, int nm, int kmax, DcWork W,
                                  const double* __restrict__ Delta_all, double* __restrict__ St_all) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (gw >= (int64_t)nm * kmax) return;
  const int mi = int(gw / kmax), i = int(gw % kmax);
  const int k = W.counts[3 * mi];
  double* St = St_all + (size_t)mi * kmax * kmax + (size_t)i * kmax;
  if (i >= k) {
    for (int j = lane; j < kmax; j += 32) St[j] = 0.0;
    return;
  }
  const double* zh = W.zh + md[mi].lo;
  const double* Delta = Delta_all + (size_t)mi * kmax * kmax + (size_t)i * k;
  double nrm = 0.0;
  for (int j = lane; j < k; j += 32) {
    const double s = zh[j] / Delta[j];
    nrm += s * s;
  }
  for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
  nrm = 1.0 / sqrt(nrm);
  for (int j = lane; j < kmax; j += 32) St[j] = (j < k) ? zh[j] / Delta[j] * nrm : 0.0;
}

// The non-deflated (rotated) columns of each block, compacted into an nbmax x kmax
// matrix per merge (zero padded); blockIdx.y = merge.
__global__ void dc_gather_kernel(const double* __restrict__ Q, int n, const MergeDesc* __restrict__ md, int nbmax,
                                 int kmax, DcWork W, double* __restrict__ Qk_all) {
  const int mi = blockIdx.y;
  const int lo = md[mi].lo, nb = md[mi].hi - lo, k = W.counts[3 * mi];
  double* Qk = Qk_all + (size_t)mi * nbmax * kmax;
  const size_t tot = (size_t)nbmax * kmax;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int r = int(e % nbmax), q = int(e / nbmax);
    double v = 0.0;
    if (r < nb && q < k) v = Q[(size_t)(lo + W.perm[lo + W.kinv[lo + q]]) * n + (lo + r)];
    Qk[e] = v;
  }
}

// Final ordering of each block (one CTA per merge): eigenvalues = roots (non-deflated)
// and deflated poles, signs undone, ascending; the source of each output column.
__global__ void dc_order_kernel(const MergeDesc* __restrict__ md, DcWork W) {
  extern __shared__ double mo_smem[];
  const int mi = blockIdx.x;
  const int lo = md[mi].lo, nb = md[mi].hi - lo;
  const int nr = W.counts[3 * mi], flip = W.counts[3 * mi + 2], nd = nb - nr;
  const bool sm = nb <= kSmemMerge;
  double* Dsm = sm ? mo_smem : W.Ds + lo;
  double* lm = sm ? Dsm + nb : W.lam + lo;
  double* wo = sm ? lm + nb : W.wn + lo;
  int* kd = sm ? (int*)(wo + nb) : W.kind + lo;
  int* sk = sm ? kd + nb : W.srck + lo;
  int* si = sm ? sk + nb : W.srci + lo;
  if (sm) {
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      Dsm[t] = W.Ds[lo + t];
      kd[t] = W.kind[lo + t];
    }
    for (int t = threadIdx.x; t < nr; t += blockDim.x) lm[t] = W.lam[lo + t];
  }
  __syncthreads();
  // the deflated slots in order (block scan), then a stable merge of the ascending roots
  // with the deflated poles (ties: the root first) by ranks on integer keys; poles moved
  // by a deflation rotation can be out of order by up to the deflation tolerance, and
  // then the merge is the serial one
  __shared__ int scan_sh[32], s_unsorted;
  int* dl = si;  // deflated slots, in the output index array until the outputs are formed
  {
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int c0 = min(nb, (int)threadIdx.x * per), c1 = min(nb, c0 + per);
    int cnt = 0;
    for (int t = c0; t < c1; ++t) cnt += 1 - kd[t];
    int tot = 0;
    int off = block_scan_excl(cnt, scan_sh, &tot);
    for (int t = c0; t < c1; ++t)
      if (!kd[t]) dl[off++] = t;
  }
  // (each thread keeps its ranks in registers: at most 16 entries of each kind)
  if (threadIdx.x == 0) s_unsorted = nb > 16 * (int)blockDim.x;
  __syncthreads();
  auto keyR = [&](int i) { return order_key(lm[i]); };
  auto keyD = [&](int j) { return order_key(Dsm[dl[j]]); };
  for (int i = threadIdx.x + 1; i < nr; i += blockDim.x)
    if (keyR(i) < keyR(i - 1)) s_unsorted = 1;
  for (int j = threadIdx.x + 1; j < nd; j += blockDim.x)
    if (keyD(j) < keyD(j - 1)) s_unsorted = 1;
  __syncthreads();
  if (!s_unsorted) {
    // ranks first (every thread reads dl), then the outputs (which overwrite si = dl)
    int posr[16], posd[16];
    int nrl = 0, ndl = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) posr[nrl++] = i + rank_in<true>(keyD, nd, keyR(i));
    for (int j = threadIdx.x; j < nd; j += blockDim.x) posd[ndl++] = j + rank_in<false>(keyR, nr, keyD(j));
    int slots[16];
    ndl = 0;
    for (int j = threadIdx.x; j < nd; j += blockDim.x) slots[ndl++] = dl[j];
    __syncthreads();
    nrl = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      const int pos = posr[nrl++], out = flip ? (nb - 1 - pos) : pos;
      sk[out] = 1;
      si[out] = i;
      wo[out] = flip ? neg_exact(lm[i]) : lm[i];
    }
    ndl = 0;
    for (int j = threadIdx.x; j < nd; j += blockDim.x) {
      const int pos = posd[ndl], slot = slots[ndl++], out = flip ? (nb - 1 - pos) : pos;
      sk[out] = 0;
      si[out] = slot;
      wo[out] = flip ? neg_exact(Dsm[slot]) : Dsm[slot];
    }
  } else if (threadIdx.x == 0) {
    int ia = 0, ib = 0, pos = 0, dslot = 0;
    while (dslot < nb && kd[dslot]) ++dslot;
    while (ia < nr || ib < nd) {
      bool takeRoot;
      if (ia >= nr)
        takeRoot = false;
      else if (ib >= nd)
        takeRoot = true;
      else
        takeRoot = lm[ia] <= Dsm[dslot];
      const int out = flip ? (nb - 1 - pos) : pos;
      if (takeRoot) {
        sk[out] = 1;
        si[out] = ia;
        wo[out] = flip ? -lm[ia] : lm[ia];
        ++ia;
      } else {
        sk[out] = 0;
        si[out] = dslot;
        wo[out] = flip ? -Dsm[dslot] : Dsm[dslot];
        ++ib;
        ++dslot;
        while (dslot < nb && kd[dslot]) ++dslot;
      }
      ++pos;
    }
  }
  __syncthreads();
  if (sm) {
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      W.srck[lo + t] = sk[t];
      W.srci[lo + t] = si[t];
      W.wn[lo + t] = wo[t];
    }
  }
}

// The merged block of every merge into T (same position as in Q): output column `out`
// is merged column srci (src kind 1) or the deflated column of Q it came from; the new
// eigenvalues into w.  blockIdx.y = merge.
__global__ void dc_scatter_kernel(const double* __restrict__ Q, int n, const MergeDesc* __restrict__ md, int nbmax,
                                  int kmax, DcWork W, const double* __restrict__ Qm_all, double* __restrict__ T,
                                  double* __restrict__ w) {
  const int mi = blockIdx.y;
  const int lo = md[mi].lo, nb = md[mi].hi - lo;
  const double* Qm = Qm_all + (size_t)mi * nbmax * kmax;
  const size_t tot = (size_t)nb * nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int r = int(e % nb), out = int(e / nb);
    const int src = W.srci[lo + out];
    const double v = W.srck[lo + out] ? Qm[r + (size_t)src * nbmax]
                                      : Q[(size_t)(lo + W.perm[lo + src]) * n + (lo + r)];
    T[(size_t)(lo + out) * n + (lo + r)] = v;
  }
  if (blockIdx.x == 0)
    for (int t = threadIdx.x; t < nb; t += blockDim.x) w[lo + t] = W.wn[lo + t];
}

// T's merged blocks back into Q; blockIdx.y = merge.
__global__ void dc_copy_kernel(const double* __restrict__ T, int n, const MergeDesc* __restrict__ md,
                               double* __restrict__ Q) {
  const int mi = blockIdx.y;
  const int lo = md[mi].lo, nb = md[mi].hi - lo;
  const size_t tot = (size_t)nb * nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t idx = (size_t)(lo + e / nb) * n + (lo + e % nb);
    Q[idx] = T[idx];
  }
}

// complex phases: T's subdiagonal is real by construction except possibly the last one
__global__ void real_to_complex_kernel(const double* Zr, int64_t rows, int64_t cols, int64_t ldr, double2* Zc,
                                       int64_t ldc) {
  size_t tot = (size_t)rows * cols;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    int64_t i = e % rows, j = e / rows;
    Zc[i + j * ldc] = make_double2(Zr[i + j * ldr], 0.0);
  }
}

__global__ void scale_rows_phase_kernel(double2* Z, int64_t rows, int64_t cols, int64_t ld, const double2* ph) {
  size_t tot = (size_t)rows * cols;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    int64_t i = e % rows, j = e / rows;
    double2 z = Z[i + j * ld], p = ph[i];
    Z[i + j * ld] = make_double2(p.x * z.x - p.y * z.y, p.x * z.y + p.y * z.x);
  }
}

// compact WY: T factors of all reflector blocks in one launch (block b = CTA b; kWY = 64
// reflectors per block, zero-padded with tau = 0) from S_b = V_b^H V_b:
// T_jj = tau_j, T[0:j, j] = -tau_j T[0:j, 0:j] S[0:j, j]; thread i owns row i; S_b and T_b
// live in shared memory.
constexpr int kWY = 64;
template <typename T>
__global__ void __launch_bounds__(kWY) wy_tfactor_kernel(const T* S, const T* tau, T* Tm) {
  extern __shared__ unsigned char wy_smem[];  // 2 x kWY x (kWY + 1) elements
  T(*Ss)[kWY + 1] = (T(*)[kWY + 1])wy_smem;
  T(*Ts)[kWY + 1] = Ss + kWY;
  const int i = threadIdx.x, b = blockIdx.x;
  const T* Sb = S + (size_t)b * kWY * kWY;
  const T* tb = tau + (size_t)b * kWY;
  T* Tb = Tm + (size_t)b * kWY * kWY;
  for (int j = 0; j < kWY; ++j) {
    Ss[i][j] = Sb[i + j * kWY];
    Ts[i][j] = czero<T>();
  }
  __syncthreads();
  for (int j = 0; j < kWY; ++j) {
    T acc = czero<T>();
    if (i < j)
      for (int l = i; l < j; ++l) acc = cadd(acc, cmulv(Ts[i][l], Ss[l][j]));
    if (i < j) Ts[i][j] = cscale(cmulv(tb[j], acc), -1.0);  // column j: read only columns < j above
    if (i == j) Ts[j][j] = tb[j];
    __syncthreads();
  }
  for (int j = 0; j < kWY; ++j) Tb[i + j * kWY] = Ts[i][j];
}

// all reflectors as the columns of an n x ncols matrix (v_kk[kk+1] = 1, zeros above,
// zero columns beyond the last reflector)
template <typename T>
__global__ void wy_extract_all_kernel(const T* A, int n, int nref, int ncols, T* V) {
  const size_t tot = (size_t)n * ncols;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int r = int(e % n), kk = int(e / n);
    T val = czero<T>();
    if (kk < nref) {
      if (r == kk + 1)
        val = cone<T>();
      else if (r > kk + 1)
        val = A[r + (size_t)kk * n];
    }
    V[e] = val;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------

struct DevBuf {
  nsg_ctx* c;
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf(nsg_ctx* cc, size_t b) : c(cc), bytes(b) { p = dalloc(c, b); }
  ~DevBuf() { dfree(c, p, bytes); }
  template <typename T>
  T* as() {
    return (T*)p;
  }
};

static void build_tree(int lo, int hi, std::vector<std::vector<MergeDesc>>& levels, std::vector<int>& leaf_lo,
                       std::vector<int>& leaf_hi, int depth, int leaf) {
  if (hi - lo <= leaf) {
    leaf_lo.push_back(lo);
    leaf_hi.push_back(hi);
    return;
  }
  int mid = lo + (hi - lo) / 2;
  build_tree(lo, mid, levels, leaf_lo, leaf_hi, depth + 1, leaf);
  build_tree(mid, hi, levels, leaf_lo, leaf_hi, depth + 1, leaf);
  if ((int)levels.size() <= depth) levels.resize(depth + 1);
  levels[depth].push_back(MergeDesc{lo, mid, hi, 0.0});
}

// Leaf order of the divide and conquer: the implicit-QL leaves are one warp each and
// latency bound (a chain of FP64 square roots and divides per rotation), so small leaves
// and more (batched) merge levels are cheaper for one solve.  The context's override
// (4..32) trades that latency for fewer levels: fewer launches and host reads.
static int dc_leaf_size(const nsg_ctx* c) { return c->tune_dc_leaf > 0 ? c->tune_dc_leaf : 8; }

// Eigen-decomposition of the real symmetric tridiagonal (d, e); Q: n x n (device,
// column-major), w: eigenvalues ascending (device).  Cuppen's divide and conquer with
// every merge of a tree level batched into one launch per step.
static void tridiag_dc(nsg_ctx* c, int n, const std::vector<double>& d_in, const std::vector<double>& e_in, double* Q,
                       double* w) {
  std::vector<std::vector<MergeDesc>> levels;
  std::vector<int> llo, lhi;
  build_tree(0, n, levels, llo, lhi, 0, dc_leaf_size(c));
  // modified diagonal: for each split subtract beta at the two touching diagonals
  std::vector<double> d = d_in;
  for (auto& lv : levels)
    for (auto& m : lv) {
      m.beta = e_in[m.mid - 1];
      d[m.mid - 1] -= m.beta;
      d[m.mid] -= m.beta;
    }
  DevBuf dd(c, sizeof(double) * n), de(c, sizeof(double) * std::max(n, 1));
  NSG_CUDA(cudaMemcpyAsync(dd.p, d.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  NSG_CUDA(cudaMemcpyAsync(de.p, e_in.data(), sizeof(double) * std::max<size_t>(e_in.size(), 1),
                           cudaMemcpyHostToDevice, c->stream));
  NSG_CUDA(cudaMemsetAsync(Q, 0, sizeof(double) * n * n, c->stream));
  // leaves
  int nleaf = int(llo.size());
  DevBuf dlo(c, sizeof(int) * nleaf), dhi(c, sizeof(int) * nleaf);
  NSG_CUDA(cudaMemcpyAsync(dlo.p, llo.data(), sizeof(int) * nleaf, cudaMemcpyHostToDevice, c->stream));
  NSG_CUDA(cudaMemcpyAsync(dhi.p, lhi.data(), sizeof(int) * nleaf, cudaMemcpyHostToDevice, c->stream));
  DevBuf lerr(c, sizeof(int));
  NSG_CUDA(cudaMemsetAsync(lerr.p, 0, sizeof(int), c->stream));
  {
    ProfScope ps(c, NSG_PROF_DC, 0.0);
    leaf_ql_kernel<<<(nleaf + kLeafWarps - 1) / kLeafWarps, 32 * kLeafWarps, 0, c->stream>>>(
        dd.as<double>(), de.as<double>(), dlo.as<int>(), dhi.as<int>(), nleaf, Q, n, w, lerr.as<int>());
  }
  count_launch(c);
  check_launch("dc leaves");
  if (levels.empty()) {
    int leaf_failed = 0;
    NSG_CUDA(cudaMemcpyAsync(&leaf_failed, lerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
    NSG_CHECK(leaf_failed == 0, NSG_ERR_NONFINITE, "eigensolver: a tridiagonal leaf did not converge");
    return;
  }
  // all levels' merge descriptors in one upload
  std::vector<MergeDesc> all;
  std::vector<size_t> off(levels.size());
  for (int L = int(levels.size()) - 1; L >= 0; --L) {
    off[L] = all.size();
    all.insert(all.end(), levels[L].begin(), levels[L].end());
  }
  DevBuf bmd(c, sizeof(MergeDesc) * all.size());
  NSG_CUDA(cudaMemcpyAsync(bmd.p, all.data(), sizeof(MergeDesc) * all.size(), cudaMemcpyHostToDevice, c->stream));
  size_t maxm = 0;
  for (auto& lv : levels) maxm = std::max(maxm, lv.size());
  DevBuf bDs(c, sizeof(double) * n), bzs(c, sizeof(double) * n), bDk(c, sizeof(double) * n),
      bzk(c, sizeof(double) * n), blam(c, sizeof(double) * n), bzh(c, sizeof(double) * n), bwn(c, sizeof(double) * n),
      brcs(c, sizeof(double) * 2 * n), bscr(c, sizeof(double) * 2 * n), bperm(c, sizeof(int) * n),
      bkind(c, sizeof(int) * n), bkinv(c, sizeof(int) * n), bsrck(c, sizeof(int) * n), bsrci(c, sizeof(int) * n),
      brpq(c, sizeof(int) * 2 * n), brho(c, sizeof(double) * maxm), bcnt(c, sizeof(int) * 3 * maxm),
      Tbuf(c, sizeof(double) * (size_t)n * n);
  DcWork W;
  W.Ds = bDs.as<double>();
  W.zs = bzs.as<double>();
  W.Dk = bDk.as<double>();
  W.zk = bzk.as<double>();
  W.lam = blam.as<double>();
  W.zh = bzh.as<double>();
  W.wn = bwn.as<double>();
  W.rot_cs = brcs.as<double>();
  W.gscr = bscr.as<double>();
  W.perm = bperm.as<int>();
  W.kind = bkind.as<int>();
  W.kinv = bkinv.as<int>();
  W.srck = bsrck.as<int>();
  W.srci = bsrci.as<int>();
  W.rot_pq = brpq.as<int>();
  W.rho = brho.as<double>();
  W.counts = bcnt.as<int>();
  std::vector<int> cnt(3 * maxm);
  bool leaves_checked = false;
  for (int L = int(levels.size()) - 1; L >= 0; --L) {
    const auto& lv = levels[L];
    const int nm = int(lv.size());
    const MergeDesc* md = bmd.as<MergeDesc>() + off[L];
    int nbmax = 0;
    for (auto& m : lv) nbmax = std::max(nbmax, m.hi - m.lo);
    {
      const int shm = nbmax <= kSmemMerge ? nbmax * 40 : 0;
      if (shm) raise_smem_limit((const void*)dc_prep_kernel, shm);
      ProfScope ps(c, NSG_PROF_DC, 0.0);
      dc_prep_kernel<<<nm, 256, shm, c->stream>>>(w, Q, n, md, W);
    }
    count_launch(c);
    check_launch("dc prep");
    NSG_CUDA(cudaMemcpyAsync(cnt.data(), W.counts, sizeof(int) * 3 * nm, cudaMemcpyDeviceToHost, c->stream));
    int leaf_failed = 0;
    if (!leaves_checked)
      NSG_CUDA(cudaMemcpyAsync(&leaf_failed, lerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
    if (!leaves_checked) {
      NSG_CHECK(leaf_failed == 0, NSG_ERR_NONFINITE, "eigensolver: a tridiagonal leaf did not converge");
      leaves_checked = true;
    }
    int kmax = 0, rotations = 0;
    for (int mi = 0; mi < nm; ++mi) {
      kmax = std::max(kmax, cnt[3 * mi]);
      rotations += cnt[3 * mi + 1];
    }
    // the deflation rotations, launched only for a level that has some (the counts are
    // on the host already for the batched product's extent)
    if (rotations > 0) {
      {
        ProfScope ps(c, NSG_PROF_DC, 0.0);
        dc_rotate_kernel<<<dim3((nbmax + 127) / 128, nm), 128, 0, c->stream>>>(Q, n, md, W);
      }
      count_launch(c);
      check_launch("dc rotate");
    }
    const int gxe = int(std::max<int64_t>(1, std::min<int64_t>(((int64_t)nbmax * nbmax + 255) / 256,
                                                                 std::max<int64_t>(1, (int64_t)c->num_sms * 8 / nm))));
    DevBuf Qm(c, sizeof(double) * (size_t)nm * nbmax * std::max(kmax, 1));
    if (kmax > 0) {
      DevBuf Delta(c, sizeof(double) * (size_t)nm * kmax * kmax), St(c, sizeof(double) * (size_t)nm * kmax * kmax),
          Qk(c, sizeof(double) * (size_t)nm * nbmax * kmax);
      const int64_t warps = (int64_t)nm * kmax;
      const int tb = 256, gb = int((warps * 32 + tb - 1) / tb);
      {
        ProfScope ps(c, NSG_PROF_DC, 0.0);
        dc_secular_kernel<<<gb, tb, 0, c->stream>>>(md, nm, kmax, W, Delta.as<double>());
        dc_gu_eisenstat_kernel<<<gb, tb, 0, c->stream>>>(md, nm, kmax, W, Delta.as<double>());
        dc_vectors_kernel<<<gb, tb, 0, c->stream>>>(md, nm, kmax, W, Delta.as<double>(), St.as<double>());
        const int gxk = int(std::max<int64_t>(
            1, std::min<int64_t>(((int64_t)nbmax * kmax + 255) / 256, std::max<int64_t>(1, (int64_t)c->num_sms * 8 / nm))));
        dc_gather_kernel<<<dim3(gxk, nm), 256, 0, c->stream>>>(Q, n, md, nbmax, kmax, W, Qk.as<double>());
      }
      count_launch(c, 4);
      check_launch("dc secular");
      GemmArgs g;
      g.dtype = NSG_F64;
      g.M = nbmax;
      g.N = kmax;
      g.K = kmax;
      g.A = Qk.p;
      g.lda = nbmax;
      g.opA = OP_N;
      g.strideA = (int64_t)nbmax * kmax;
      g.B = St.p;
      g.ldb = kmax;
      g.opB = OP_N;
      g.strideB = (int64_t)kmax * kmax;
      g.C = Qm.p;
      g.ldc = nbmax;
      g.strideC = (int64_t)nbmax * kmax;
      g.batch = nm;
      gemm_accurate(c, g);
    }
    {
      const int shm = nbmax <= kSmemMerge ? nbmax * 36 : 0;
      if (shm) raise_smem_limit((const void*)dc_order_kernel, shm);
      ProfScope ps(c, NSG_PROF_DC, 0.0);
      dc_order_kernel<<<nm, 256, shm, c->stream>>>(md, W);
      dc_scatter_kernel<<<dim3(gxe, nm), 256, 0, c->stream>>>(Q, n, md, nbmax, std::max(kmax, 1), W, Qm.as<double>(),
                                                             Tbuf.as<double>(), w);
      dc_copy_kernel<<<dim3(gxe, nm), 256, 0, c->stream>>>(Tbuf.as<double>(), n, md, Q);
    }
    count_launch(c, 3);
    check_launch("dc merge");
  }
}

template <typename T>
static void back_transform(nsg_ctx* c, int dtype, int n, const T* A, const T* tau_dev, T* Z, int64_t ldz, int64_t k) {
  // Z <- H_0 H_1 ... H_{n-3} Z in blocks of kWY reflectors, last block first.  Every
  // block's V, S = V^H V and T factor are formed up front (one launch each); the
  // sequential part is then three GEMMs per block.
  const int nref = n - 2;
  if (nref <= 0 || k == 0) return;
  const int NB = kWY, nblk = (nref + NB - 1) / NB, ncols = nblk * NB;
  const size_t eb = sizeof(T);
  DevBuf V(c, eb * (size_t)n * ncols), S(c, eb * (size_t)NB * NB * nblk), Tm(c, eb * (size_t)NB * NB * nblk),
      taup(c, eb * ncols), Wt(c, eb * (size_t)NB * k), W2(c, eb * (size_t)NB * k);
  {
    int gblocks = int(std::min<size_t>(((size_t)n * ncols + 255) / 256, (size_t)c->num_sms * 8));
    wy_extract_all_kernel<T><<<gblocks, 256, 0, c->stream>>>(A, n, nref, ncols, V.as<T>());
    NSG_CUDA(cudaMemsetAsync(taup.p, 0, eb * ncols, c->stream));
    NSG_CUDA(cudaMemcpyAsync(taup.p, tau_dev, eb * nref, cudaMemcpyDeviceToDevice, c->stream));
    count_launch(c);
  }
  // S_b = V_b^H V_b over all n rows (rows above a block's reflectors are zero)
  GemmArgs g;
  g.dtype = dtype;
  g.M = NB;
  g.N = NB;
  g.K = n;
  g.A = V.p;
  g.lda = n;
  g.opA = OP_C;
  g.strideA = (int64_t)n * NB;
  g.B = V.p;
  g.ldb = n;
  g.opB = OP_N;
  g.strideB = (int64_t)n * NB;
  g.C = S.p;
  g.ldc = NB;
  g.strideC = (int64_t)NB * NB;
  g.batch = nblk;
  gemm_f64_simt(c, g);
  {
    const int shm = int(2 * NB * (NB + 1) * eb);
    raise_smem_limit((const void*)wy_tfactor_kernel<T>, shm);
    wy_tfactor_kernel<T><<<nblk, NB, shm, c->stream>>>(S.as<T>(), taup.as<T>(), Tm.as<T>());
  }
  count_launch(c);
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * NB, nbk = std::min(NB, nref - k0), rows = n - (k0 + 1);
    const T* Vb = V.as<T>() + (k0 + 1) + (size_t)k0 * n;
    // W = V_b^H Z(rows k0+1..)  (nbk x k)
    GemmArgs h;
    h.dtype = dtype;
    h.batch = 1;
    h.strideA = h.strideB = h.strideC = 0;
    h.M = nbk;
    h.N = k;
    h.K = rows;
    h.A = Vb;
    h.lda = n;
    h.opA = OP_C;
    h.B = Z + (k0 + 1);
    h.ldb = ldz;
    h.opB = OP_N;
    h.C = Wt.p;
    h.ldc = nbk;
    gemm_accurate(c, h);
    // W2 = T_b W
    GemmArgs t2 = h;
    t2.M = nbk;
    t2.N = k;
    t2.K = nbk;
    t2.A = Tm.as<T>() + (size_t)b * NB * NB;
    t2.lda = NB;
    t2.opA = OP_N;
    t2.B = Wt.p;
    t2.ldb = nbk;
    t2.opB = OP_N;
    t2.C = W2.p;
    t2.ldc = nbk;
    gemm_f64_simt(c, t2);
    // Z -= V_b W2
    GemmArgs u = h;
    u.M = rows;
    u.N = k;
    u.K = nbk;
    u.A = Vb;
    u.lda = n;
    u.opA = OP_N;
    u.B = W2.p;
    u.ldb = nbk;
    u.opB = OP_N;
    u.C = Z + (k0 + 1);
    u.ldc = ldz;
    u.alpha_re = -1.0;
    u.beta_re = 1.0;
    gemm_accurate(c, u);
  }
  check_launch("back_transform");
}

// Cluster tridiagonalisation when the matrix fits the distributed shared memory of one
// cluster (up to 16 CTAs of ~200 KB).  The cluster size comes from the tuning table by
// order (measured: the reduction is FP64-bound on its C SMs, and a CTA's remote reads
// per step do not grow with C; orders above the table take the grid kernel), or from the
// context's override; it is raised until the columns fit.  Returns false (nothing
// launched) for the grid kernel or when no cluster shape fits.
template <typename T>
static bool tridiag_cluster(nsg_ctx* c, int n, T* A, double* d, double* e, T* tau) {
  if (n < 3 || c->tune_tri == -1) return false;
  const size_t eb = sizeof(T);
  int C = c->tune_tri;
  if (C == 0) {
    for (const auto& t : tuning::kTri)
      if (n <= t.max_order) {
        C = t.path;
        break;
      }
    if (C == 0) return false;
  }
  auto kfn = tridiag_cluster_kernel<T>;
  for (; C <= 16; C *= 2) {
    const size_t ncol = (size_t(n) + C - 1) / C;
    const size_t smem = (ncol * n + 4 * size_t(n)) * eb;
    if (smem > 200 * 1024) continue;
    ensure_smem_limit((const void*)kfn, int(smem));
    if (C > 8) NSG_CUDA(cudaFuncSetAttribute((const void*)kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kClusterTriThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)kfn, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    ProfScope ps(c, NSG_PROF_TRIDIAG, (sizeof(T) == 16 ? 16.0 : 4.0) / 3.0 * double(n) * n * n);
    NSG_CUDA(cudaLaunchKernelEx(&cfg, kfn, A, n, d, e, tau));
    count_launch(c);
    check_launch("tridiag (cluster)");
    return true;
  }
  return false;
}

// Hermitian eigen-decomposition of A (n x n, consumed).  Eigenvalues ascending into
// w_host; eigenvectors for the eigenvalue indices `cols` (ascending order indices)
// into Zout (n x ncols, column-major).  The caller chooses cols after seeing the
// spectrum through `pick`.
template <typename T>
static void syevd_dc_impl(nsg_ctx* c, int dtype, int n, T* A, std::vector<double>& w_host, const PickFn& pick) {
  const size_t eb = sizeof(T);
  DevBuf dd(c, sizeof(double) * n), de(c, sizeof(double) * std::max(n, 1)), dtau(c, eb * std::max(n, 1));
  NSG_CUDA(cudaMemsetAsync(dtau.p, 0, eb * std::max(n, 1), c->stream));
  std::vector<double> d(n), e(std::max(n - 1, 0));
  if (n == 1) {
    T a;
    NSG_CUDA(cudaMemcpyAsync(&a, A, eb, cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
    d[0] = ((double*)&a)[0];
  } else if (tridiag_cluster<T>(c, n, A, dd.as<double>(), de.as<double>(), dtau.as<T>())) {
    NSG_CUDA(cudaMemcpyAsync(d.data(), dd.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaMemcpyAsync(e.data(), de.p, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
  } else {
    // cooperative tridiagonalisation
    int max_blocks = 0;
    size_t shm = eb * 3 * n;
    NSG_CHECK(shm <= 200 * 1024, NSG_ERR_UNSUPPORTED, "tridiagonalisation: matrix order too large");
    // one CTA per SM: the active CTAs (the first nact block indices) are then spread over
    // all SMs.  256 threads (two warps per SM sub-partition) for real data, 128 for complex
    // data (measured: 128 threads 17 % slower for real, 6 % faster for complex at n = 1024;
    // 512 threads and two CTAs per SM slower for both)
    constexpr int kTriThreads = sizeof(T) == 8 ? 256 : 128;
    auto kfn = tridiag_kernel<T, kTriThreads>;
    raise_smem_limit((const void*)kfn, int(shm));
    NSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_blocks, kfn, kTriThreads, shm));
    NSG_CHECK(max_blocks > 0, NSG_ERR_UNSUPPORTED, "tridiagonalisation: no resident block fits");
    int64_t want = ((int64_t)n * n + kTriThreads * 8 - 1) / (kTriThreads * 8);
    int grid = int(std::min<int64_t>({(int64_t)max_blocks * c->num_sms, std::max<int64_t>(want, 1),
                                      (int64_t)c->num_sms}));
    {
      const int64_t rb = sizeof(T) == 8 ? 512 : 256, m = n - 1;
      const int64_t units = ((m + grid - 1) / grid) * ((m + rb - 1) / rb);
      NSG_CHECK(units <= kTriUnits, NSG_ERR_UNSUPPORTED, "tridiagonalisation: matrix order too large for the grid");
    }
    DevBuf xbuf(c, eb * 2 * n), part(c, sizeof(double2) * 2 * grid), bar(c, sizeof(Barrier));
    NSG_CUDA(cudaMemsetAsync(bar.p, 0, sizeof(Barrier), c->stream));
    double* pd = dd.as<double>();
    double* pe = de.as<double>();
    T* pt = dtau.as<T>();
    T* px = xbuf.as<T>();
    T* pp = part.as<T>();
    Barrier* pb = bar.as<Barrier>();
    int pt_arg = 1024 / kTriThreads;  // trailing elements per thread before another CTA joins the pass
    void* args[] = {&A, &n, &pd, &pe, &pt, &px, &pp, &pb, &pt_arg};
    ProfScope ps(c, NSG_PROF_TRIDIAG, (sizeof(T) == 16 ? 16.0 : 4.0) / 3.0 * double(n) * n * n);
    NSG_CUDA(cudaLaunchCooperativeKernel((void*)kfn, dim3(grid), dim3(kTriThreads), args, shm,
                                         c->stream));
    count_launch(c);
    check_launch("tridiag");
    Barrier hb;
    NSG_CUDA(cudaMemcpyAsync(&hb, bar.p, sizeof(Barrier), cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaMemcpyAsync(d.data(), dd.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaMemcpyAsync(e.data(), de.p, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, c->stream));
    NSG_CUDA(cudaStreamSynchronize(c->stream));
    NSG_CHECK(hb.err == 0, NSG_ERR_TIMEOUT, "tridiagonalisation: grid barrier timed out");
  }
  std::vector<double2> phase(n, make_double2(1.0, 0.0));
  if constexpr (sizeof(T) == 16) {
    // the last subdiagonal entry A[n-1, n-2] may be complex: make it real with a phase on row n-1
    if (n >= 2) {
      double2 last;
      NSG_CUDA(cudaMemcpyAsync(&last, (double2*)A + (n - 1) + (size_t)(n - 2) * n, sizeof(double2),
                               cudaMemcpyDeviceToHost, c->stream));
      NSG_CUDA(cudaStreamSynchronize(c->stream));
      double r = std::hypot(last.x, last.y);
      e[n - 2] = r;
      if (r > 0) phase[n - 1] = make_double2(last.x / r, last.y / r);
    }
  }
  for (double x : d) NSG_CHECK(std::isfinite(x), NSG_ERR_NONFINITE, "eigensolver: non-finite tridiagonal");
  for (double x : e) NSG_CHECK(std::isfinite(x), NSG_ERR_NONFINITE, "eigensolver: non-finite tridiagonal");
  DevBuf Q(c, sizeof(double) * (size_t)n * n), wdev(c, sizeof(double) * n);
  if (n == 1) {
    double one = 1.0;
    NSG_CUDA(cudaMemcpyAsync(Q.p, &one, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    NSG_CUDA(cudaMemcpyAsync(wdev.p, d.data(), sizeof(double), cudaMemcpyHostToDevice, c->stream));
  } else {
    tridiag_dc(c, n, d, e, Q.as<double>(), wdev.as<double>());
  }
  w_host.resize(n);
  NSG_CUDA(cudaMemcpyAsync(w_host.data(), wdev.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  for (double x : w_host) NSG_CHECK(std::isfinite(x), NSG_ERR_NONFINITE, "eigensolver: non-finite eigenvalue");
  void* Zv = nullptr;
  int64_t ldz = 0;
  std::vector<int> cols = pick(w_host, &Zv, &ldz);
  T* Zout = (T*)Zv;
  int64_t kc = int64_t(cols.size());
  if (kc == 0) return;
  // gather the chosen tridiagonal eigenvectors into Zout (real -> T)
  DevBuf didx(c, sizeof(int) * kc);
  NSG_CUDA(cudaMemcpyAsync(didx.p, cols.data(), sizeof(int) * kc, cudaMemcpyHostToDevice, c->stream));
  if constexpr (sizeof(T) == 8) {
    copy_columns(c, NSG_F64, n, kc, Q.p, n, didx.as<int>(), Zout, ldz);
  } else {
    DevBuf Zr(c, sizeof(double) * (size_t)n * kc);
    copy_columns(c, NSG_F64, n, kc, Q.p, n, didx.as<int>(), Zr.p, n);
    int gblocks = int(std::min<size_t>(((size_t)n * kc + 255) / 256, (size_t)c->num_sms * 8));
    real_to_complex_kernel<<<gblocks, 256, 0, c->stream>>>(Zr.as<double>(), n, kc, n, (double2*)Zout, ldz);
    DevBuf ph(c, sizeof(double2) * n);
    NSG_CUDA(cudaMemcpyAsync(ph.p, phase.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
    scale_rows_phase_kernel<<<gblocks, 256, 0, c->stream>>>((double2*)Zout, n, kc, ldz, ph.as<double2>());
    count_launch(c, 2);
  }
  back_transform<T>(c, dtype, n, A, dtau.as<T>(), Zout, ldz, kc);
}

void syevd_dc(nsg_ctx* c, int dtype, int n, void* A, std::vector<double>& w_host, const PickFn& pick) {
  if (dtype == NSG_C128)
    syevd_dc_impl<double2>(c, dtype, n, (double2*)A, w_host, pick);
  else
    syevd_dc_impl<double>(c, dtype, n, (double*)A, w_host, pick);
}

}  // namespace nsg
