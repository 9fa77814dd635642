/*
 * nsg.h — C ABI of the GB300 sweep kernels for NetworkSolvers.jl.
 *
 * Every numerical step under the reference's plugin functions is reached through
 * these entry points; the Julia (or Python) side keeps the drivers, region plans and
 * problem types and holds opaque device handles.  Plain C types only; no exceptions
 * cross this boundary; every call returns an `NSG_*` status and `nsg_last_error`
 * gives the message.  All work is ordered on the context's CUDA stream; calls that
 * return scalars (eigenvalue, kept bond dimension, truncation error, norms)
 * synchronise that stream before returning.
 *
 * Layout contract: a tensor of rank r with dims (d0, ..., d{r-1}) is dense and
 * column-major (d0 fastest) — the memory layout of an ITensor whose indices are in
 * that order.  State tensors arrive with the index order fixed by
 * permute_indices.jl:4-18 ([first link, site(s), other links]).
 *
 * Indices are named by int32 labels chosen by the caller (ITensor index ids with
 * prime levels map to distinct labels).  Labels shared by two tensors are summed.
 *
 * Reference interfaces replaced (paths within emstoudenmire/NetworkSolvers.jl):
 *   optimal_map(P::ProjTTN, ψ)          operator_map.jl:3-10   -> nsg_linmap_*, nsg_contract
 *   ProjTTN environment update          extracter.jl:14        -> nsg_contract
 *   local_state = prod(ψ[v] for region) extracter.jl:7         -> nsg_contract
 *   eigsolve_solver (KrylovKit Lanczos) local_solvers/eigsolve.jl:3-29  -> nsg_eigsolve
 *   exponentiate_solver (KrylovKit)     local_solvers/exponentiate.jl:3-29 -> nsg_exponentiate
 *   runge_kutta_solver                  local_solvers/runge_kutta.jl:16-25 -> nsg_runge_kutta
 *   it.factorize(local, indsTe; trunc)  inserter.jl:23         -> nsg_factorize
 *   qr (gauge walk / 1-site TDVP)       extracter.jl:6, applyexp.jl:37 -> nsg_qr
 *   eigen(rho; trunc, ishermitian)      subspace/densitymatrix.jl:53 -> nsg_eigh
 *   directsum(A=>a, U=>u)               subspace/densitymatrix.jl:64 -> nsg_concat
 *   norm / normalize / (T - P*T)        inserter.jl:31, densitymatrix.jl:48-59 -> nsg_norm, nsg_axpby, nsg_dot
 */
#ifndef NSG_H
#define NSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define NSG_OK 0
#define NSG_ERR_INVALID 1        /* bad argument, shape or label set        */
#define NSG_ERR_OOM 2            /* allocation beyond the context's budget  */
#define NSG_ERR_CUDA 3           /* CUDA runtime error                      */
#define NSG_ERR_NONFINITE 4      /* NaN/Inf in a scalar result              */
#define NSG_ERR_NOT_CONVERGED 5  /* iteration limit reached                 */
#define NSG_ERR_TIMEOUT 6        /* a bounded device-side wait gave up      */
#define NSG_ERR_UNSUPPORTED 7

/* ---- element types and precision modes ---------------------------------- */
#define NSG_F64 0                /* real double                             */
#define NSG_C128 1               /* complex double (re, im interleaved)     */

#define NSG_PREC_FP64 0          /* every contraction in FP64 on the CUDA cores           */
#define NSG_PREC_TF32X3 1        /* large contractions: 3 TF32 products, FP32 accumulate  */
#define NSG_PREC_OZAKI 2         /* large contractions: 6 BF16 slices per operand, 21
                                    products, exact FP32 accumulation per 128-deep chunk:
                                    1e-12-level accuracy on the tensor cores             */
#define NSG_PREC_OZAKI8 3        /* as NSG_PREC_OZAKI with 8 slices (36 products): FP64
                                    accuracy (2^-55 of the row and column scales)        */

#define NSG_MAX_RANK 16

typedef struct nsg_ctx nsg_ctx;
typedef struct nsg_tensor nsg_tensor;
typedef struct nsg_linmap nsg_linmap;

/* ---- context --------------------------------------------------------------
 * One context per host thread; it owns a CUDA stream, a stream-ordered device
 * memory pool capped at `hbm_budget_bytes` (0 = no cap) and scratch buffers. */
int nsg_ctx_create(int device, uint64_t hbm_budget_bytes, nsg_ctx** out);
int nsg_ctx_destroy(nsg_ctx* ctx);
const char* nsg_last_error(const nsg_ctx* ctx);
int nsg_ctx_set_precision(nsg_ctx* ctx, int precision);
int nsg_ctx_synchronize(nsg_ctx* ctx);
/* bytes in use / peak / budget */
int nsg_ctx_memory(const nsg_ctx* ctx, uint64_t* in_use, uint64_t* peak, uint64_t* budget);
/* Free and total device memory of `device` (cudaMemGetInfo): the admission budget of a
   pool of concurrent solves.  No counterpart in the reference (single solve per process). */
int nsg_device_memory(int device, uint64_t* free_bytes, uint64_t* total_bytes);
/* counters[0] = kernel launches, [1] = algorithmic flops of contractions,
 * [2] = contraction calls, [3] = linear-map applications; reset if `reset`. */
int nsg_ctx_counters(nsg_ctx* ctx, uint64_t* counters4, int reset);

/* Device-side timing on the context's stream: record event `slot` (0..15); elapsed
 * milliseconds between two recorded slots (synchronises on the later one). */
int nsg_ctx_event_record(nsg_ctx* ctx, int slot);
int nsg_ctx_event_elapsed(nsg_ctx* ctx, int slot_from, int slot_to, float* ms);
/* Per-kernel-class profiling: while enabled, launches of the classes below are
 * bracketed by CUDA events on the context's stream.  Reading synchronises and returns
 * the launch count, the summed device milliseconds and the summed algorithmic flops
 * (real flops; for tensor-core GEMMs the FP64-equivalent 2*M*N*K). Enabling resets. */
#define NSG_PROF_TC_GEMM 0     /* tcgen05 split-precision GEMM kernel              */
#define NSG_PROF_SPLIT 1       /* FP64 -> TF32 slice pass                          */
#define NSG_PROF_SIMT_GEMM 2   /* FP64 CUDA-core GEMM                              */
#define NSG_PROF_TRIDIAG 3     /* Householder tridiagonalisation                   */
#define NSG_PROF_DC 4          /* divide and conquer: leaves, merges, secular roots */
#define NSG_PROF_NCLASS 5
int nsg_ctx_profile(nsg_ctx* ctx, int enable);
int nsg_ctx_profile_read(nsg_ctx* ctx, int cls, uint64_t* launches, double* ms, double* flops);

/* Per-phase timers of the region step (the reference's timed examples wrap each plugin
 * in @elapsed; here the device time on the context's stream).  While enabled
 * (nsg_ctx_timers), the host brackets the phases of a region step with
 * nsg_ctx_phase(ctx, phase, 1) ... nsg_ctx_phase(ctx, phase, 0), which record CUDA events
 * on the context's stream, and the library brackets every linear-map application
 * (NSG_PHASE_HEFF) and the phases of nsg_region_step itself.  nsg_get_timers synchronises
 * and returns per phase the number of closed intervals and their summed device
 * milliseconds (arrays of NSG_PHASE_NCOUNT).  Phases may nest (H_eff inside Krylov, the
 * expansion inside extraction); a phase may not be opened twice.  Enabling resets. */
#define NSG_PHASE_EXTRACT 0   /* gauge walk, region product, environment updates  */
#define NSG_PHASE_SUBSPACE 1  /* density-matrix subspace expansion                */
#define NSG_PHASE_KRYLOV 2    /* local solver: eigsolve / exponentiate / Runge-Kutta */
#define NSG_PHASE_HEFF 3      /* linear-map (H_eff) applications                  */
#define NSG_PHASE_FACTORIZE 4 /* truncated factorization of the inserter          */
#define NSG_PHASE_NCOUNT 5
int nsg_ctx_timers(nsg_ctx* ctx, int enable);
int nsg_ctx_phase(nsg_ctx* ctx, int phase, int begin);
int nsg_get_timers(nsg_ctx* ctx, uint64_t* counts, double* ms);

/* Diagnostic of the timeout path (no counterpart in the reference): launches a kernel
 * that waits on the context's stream, with the bounded pattern of the library's own
 * device waits, for a device flag that nothing sets.  After `polls` polls (1..2^24, each
 * about 0.1 us) the wait gives up, raises the context's error flag and the call returns
 * NSG_ERR_TIMEOUT; the context stays usable.  Hosts use it to check that they turn
 * that status into an error. */
int nsg_ctx_wait_probe(nsg_ctx* ctx, int64_t polls);

/* Launch-choice override of this context, for the autotuner that writes the library's
 * compiled-in tuning table (no counterpart in the reference).  param NSG_TUNE_SPLITK:
 * number of K slices of the FP64 CUDA-core GEMM (1..64; 0 restores the table);
 * NSG_TUNE_TRIDIAG: the Householder tridiagonalisation's path (-1 the grid-wide kernel,
 * 2/4/8/16 one thread-block cluster of that size where the matrix fits it, 0 the table);
 * NSG_TUNE_DC_LEAF: the divide and conquer's leaf order (4..32; 0 the default 8: larger
 * leaves mean fewer merge levels, so fewer launches and host reads per eigensolve, at a
 * longer leaf solve; a throughput choice for many concurrent small solves). */
#define NSG_TUNE_SPLITK 0
#define NSG_TUNE_TRIDIAG 1
#define NSG_TUNE_DC_LEAF 2
int nsg_ctx_set_tuning(nsg_ctx* ctx, int param, int value);

/* ---- tensors ------------------------------------------------------------- */
int nsg_tensor_create(nsg_ctx* ctx, int dtype, int rank, const int64_t* dims, nsg_tensor** out);
int nsg_tensor_upload(nsg_ctx* ctx, int dtype, int rank, const int64_t* dims,
                      const void* host, nsg_tensor** out);
int nsg_tensor_download(nsg_ctx* ctx, const nsg_tensor* t, void* host);
int nsg_tensor_release(nsg_ctx* ctx, nsg_tensor* t);
int nsg_tensor_shape(const nsg_tensor* t, int* dtype, int* rank, int64_t* dims);
int nsg_tensor_copy(nsg_ctx* ctx, const nsg_tensor* src, nsg_tensor** out);
/* device pointer (for callers that share device memory, e.g. torch) */
int nsg_tensor_device_ptr(const nsg_tensor* t, void** ptr);

/* ---- vector algebra on equally shaped tensors ---------------------------- */
/* y = a*x + b*y (complex scalars given as re/im pairs; ignored im for F64) */
int nsg_axpby(nsg_ctx* ctx, double a_re, double a_im, const nsg_tensor* x,
              double b_re, double b_im, nsg_tensor* y);
/* <x, y> = sum conj(x) y */
int nsg_dot(nsg_ctx* ctx, const nsg_tensor* x, const nsg_tensor* y, double* re, double* im);
int nsg_norm(nsg_ctx* ctx, const nsg_tensor* x, double* out);
/* permute axes: out axis k = in axis perm[k]; optional complex conjugation */
int nsg_permute(nsg_ctx* ctx, const nsg_tensor* x, const int* perm, int conj, nsg_tensor** out);
/* concatenate along `axis` (all other dims equal)  — ITensors directsum */
int nsg_concat(nsg_ctx* ctx, const nsg_tensor* a, const nsg_tensor* b, int axis, nsg_tensor** out);
/* dst(r0d + i, c0d + j) = src(r0s + i, c0s + j) (accumulate != 0: +=) for i < rows, j < cols,
 * each tensor's column-major storage viewed as a matrix with leading dimension lds / ldd;
 * the boxes must lie inside both tensors.  The block-sparse (QN) layer assembles the
 * sector matrices of its factorizations and cuts its blocks back out with it (NDTensors
 * BlockSparse storage: per-block dense data placed at block offsets). */
int nsg_copy_submatrix(nsg_ctx* ctx, const nsg_tensor* src, int64_t lds, int64_t r0s, int64_t c0s,
                       nsg_tensor* dst, int64_t ldd, int64_t r0d, int64_t c0d, int64_t rows, int64_t cols,
                       int accumulate);

/* ---- contraction ---------------------------------------------------------
 * Contract n tensors; tensor k has rank r_k (its own rank) and labels
 * labels[off_k .. off_k + r_k) with off_k = sum of earlier ranks; conj[k] != 0
 * conjugates tensor k.  Labels appearing twice are summed; the result has
 * `out_rank` axes with labels `out_labels` (each appearing exactly once among the
 * inputs).  The pairwise order minimises flops (exhaustive over subsets). */
int nsg_contract(nsg_ctx* ctx, int n, nsg_tensor* const* tensors, const int32_t* labels,
                 const int* conj, int out_rank, const int32_t* out_labels, nsg_tensor** out);

/* A linear map y = M x built from fixed tensors and one vector slot (H_eff of
 * optimal_map).  x has labels x_labels (x_rank of them); the result's axis k is the
 * label y_labels[k] and is stored in x's shape (noprime).  Fixed-only parts of the
 * contraction order are evaluated once at creation. */
int nsg_linmap_create(nsg_ctx* ctx, int n_fixed, nsg_tensor* const* fixed,
                      const int32_t* labels, const int* conj, int x_rank,
                      const int32_t* x_labels, const int32_t* y_labels, nsg_linmap** out);
int nsg_linmap_apply(nsg_ctx* ctx, nsg_linmap* m, const nsg_tensor* x, nsg_tensor* y);
int nsg_linmap_release(nsg_ctx* ctx, nsg_linmap* m);
/* flops of one application (algorithmic, real flops; complex MAC = 8) */
int nsg_linmap_flops(const nsg_linmap* m, double* flops);

/* ---- local solvers ------------------------------------------------------- */
/* Lowest eigenpair (Lanczos, full reorthogonalisation).  x: initial vector in,
 * normalised Ritz vector out. */
int nsg_eigsolve(nsg_ctx* ctx, nsg_linmap* m, nsg_tensor* x, int krylovdim, int maxiter,
                 double tol, double* eigval, int* numops);
/* x <- exp(t M) x for Hermitian M, t complex (Lanczos exponential integrator). */
int nsg_exponentiate(nsg_ctx* ctx, nsg_linmap* m, double t_re, double t_im, nsg_tensor* x,
                     int krylovdim, int maxiter, double tol, int* converged, int* numops);
/* x <- RK2/RK4 step of dx/dt = M x over t (runge_kutta.jl:2-14 algebra). */
int nsg_runge_kutta(nsg_ctx* ctx, nsg_linmap* m, double t_re, double t_im, nsg_tensor* x,
                    int order);

/* ---- factorizations -------------------------------------------------------
 * Matrix view: rows = axes left_axes[0..n_left) of T (in that order), columns = the
 * remaining axes in storage order.  Singular values / eigenvalues are truncated by
 * the NDTensors rule (relative discarded weight `cutoff`, `maxdim`, `mindim`;
 * maxdim <= 0 means unlimited).  U: [left dims..., k], C: [k, right dims...]. */
int nsg_factorize(nsg_ctx* ctx, const nsg_tensor* T, const int* left_axes, int n_left,
                  double cutoff, int64_t maxdim, int64_t mindim, nsg_tensor** U,
                  nsg_tensor** C, int64_t* newdim, double* truncerr, double* spectrum,
                  int64_t spectrum_cap);
/* nsg_factorize (no spectrum) that also returns, in *Uperp, an orthonormal basis
 * [left dims..., rows - k] of the complement of U's columns in the row space when the
 * factorization went through the row-side Gram matrix M M^H (the discarded
 * eigenvectors), NULL otherwise (the narrow-side route for tall M, or k = rows).  The
 * densitymatrix expansion of the next region (subspace/densitymatrix.jl:44-59) works in
 * this complement: its eigen(rho) restricted to it is the same eigenproblem. */
int nsg_factorize_complement(nsg_ctx* ctx, const nsg_tensor* T, const int* left_axes, int n_left,
                             double cutoff, int64_t maxdim, int64_t mindim, nsg_tensor** U,
                             nsg_tensor** C, nsg_tensor** Uperp, int64_t* newdim, double* truncerr);
/* Q: [left dims..., k], R: [k, right dims...], k = min(rows, cols). */
int nsg_qr(nsg_ctx* ctx, const nsg_tensor* T, const int* left_axes, int n_left,
           nsg_tensor** Q, nsg_tensor** R);
/* Hermitian eigen of rho viewed as (rows = axes row_axes) x (remaining axes), which
 * must be the same space; eigenvalues descending, truncated.  U: [col dims..., k]
 * (eigenvectors on the column space, the unprimed kets), evals: first k values. */
int nsg_eigh(nsg_ctx* ctx, const nsg_tensor* rho, const int* row_axes, int n_row,
             double cutoff, int64_t maxdim, int64_t mindim, nsg_tensor** U,
             double* evals, int64_t evals_cap, int64_t* newdim, double* truncerr);

/* ---- fused region step ----------------------------------------------------
 * One two-site DMRG region step on a chain in one call (the extracter product,
 * extracter.jl:7; the Lanczos updater, eigsolve.jl:14-28; the truncated-factorization
 * inserter, inserter.jl:3-33), composed of the entry points above:
 *   L [a', wl, a], W1 [wl, s1', s1, wm], W2 [wm, s2', s2, wr], R [b', wr, b] (the fixed
 *   tensors of optimal_map, operator_map.jl:3-10), psi1 [a, s1, c], psi2 [c, s2, b].
 * Outputs: the new site tensors left [a, s1, k] and right [k, s2, b], the Lanczos
 * eigenvalue, the new bond dimension k and the relative discarded weight.  direction 0
 * (region (v1, v2) of a left-to-right pass): left = U is left-orthonormal, right = C;
 * direction 1 (region (v2, v1) of a right-to-left pass): right = U is right-orthonormal,
 * left = C (inserter.jl:23 factorizes on the indices of the region's first vertex). */
int nsg_region_step(nsg_ctx* ctx, nsg_tensor* L, nsg_tensor* W1, nsg_tensor* W2, nsg_tensor* R,
                    const nsg_tensor* psi1, const nsg_tensor* psi2, int direction, int krylovdim,
                    int maxiter, double tol, double cutoff, int64_t maxdim, int64_t mindim,
                    nsg_tensor** left, nsg_tensor** right, double* energy, int64_t* newdim,
                    double* truncerr);

/* ---- allocation-free GEMM -------------------------------------------------
 * No counterpart in the reference: an addition for callers that must not allocate
 * device memory themselves (a Julia program whose CUDA.jl memory pool owns the device,
 * a host whose caching allocator must account for every byte, a latency-bound caller
 * that cannot absorb the synchronisation of cudaMalloc/cudaFree).
 *
 * C = alpha op(A) op(B) + beta C in the TF32x3 split-precision form of the tensor-core
 * contractions, for real FP64 column-major matrices already on the current device;
 * op(X) = X^T when trans* != 0.  Work is ordered on `stream` (NULL = legacy default
 * stream) and the call synchronises it before returning.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: the operand slices and the device error
 * flag live in one static device array of 64 MiB (plus a 256-byte header), held by
 * every GPU that loads the library until the process exits; sizes whose padded slices
 * exceed it (or any extent above 2^23) are rejected with NSG_ERR_UNSUPPORTED.  The
 * first call on a device resolves that array's address and configures the kernel (with
 * the device current).  Every call synchronises `stream` and reads the error flag back
 * into host memory, so the entry point cannot be called while `stream` is being
 * captured into a CUDA graph.  All calls share the array: calls that overlap on the GPU
 * (other streams, other threads) race on it.  On failure the
 * message is written to errbuf (errlen bytes, NUL-terminated). */
int nsg_gemm_tf32x3_noalloc(const double* A, int64_t lda, int transA, const double* B, int64_t ldb,
                            int transB, double* C, int64_t ldc, int64_t M, int64_t N, int64_t K,
                            double alpha, double beta, void* stream, char* errbuf, int errlen);

#ifdef __cplusplus
}
#endif
#endif /* NSG_H */
