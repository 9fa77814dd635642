// Context, device memory pool, tensor handles and the vector-algebra entry points.
#include "nsg_internal.h"

#include <cstring>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>

namespace nsg {

void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(NSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void bind_device(const nsg_ctx* c) {
  if (!c) return;
  int cur = -1;
  NSG_CUDA(cudaGetDevice(&cur));
  if (cur != c->device) NSG_CUDA(cudaSetDevice(c->device));
}

void ensure_smem_limit(const void* fn, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> limit;
  int dev = 0;
  NSG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(mu);
  int& cur = limit[{dev, fn}];
  if (bytes <= cur) return;
  NSG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  cur = bytes;
}

void* dalloc(nsg_ctx* c, size_t bytes) {
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) & ~size_t(255);
  if (c->budget && c->in_use + bytes > c->budget)
    throw Error(NSG_ERR_OOM, "allocation of " + std::to_string(bytes) + " bytes exceeds the HBM budget (" +
                                 std::to_string(c->in_use) + " of " + std::to_string(c->budget) + " in use)");
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(NSG_ERR_OOM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  }
  c->in_use += bytes;
  if (c->in_use > c->peak) c->peak = c->in_use;
  return p;
}

void dfree(nsg_ctx* c, void* p, size_t bytes) {
  if (!p) return;
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) & ~size_t(255);
  NSG_CUDA(cudaFreeAsync(p, c->stream));
  c->in_use -= bytes;
}

nsg_tensor* new_tensor(nsg_ctx* c, int dtype, int rank, const int64_t* dims, bool zero) {
  NSG_CHECK(dtype == NSG_F64 || dtype == NSG_C128, NSG_ERR_INVALID, "unknown dtype");
  NSG_CHECK(rank >= 0 && rank <= NSG_MAX_RANK, NSG_ERR_INVALID, "rank out of range");
  auto* t = new nsg_tensor();
  t->dtype = dtype;
  t->rank = rank;
  t->size = 1;
  for (int k = 0; k < rank; ++k) {
    NSG_CHECK(dims[k] >= 1, NSG_ERR_INVALID, "tensor dimensions must be >= 1");
    t->dims[k] = dims[k];
    t->size *= dims[k];
  }
  t->bytes = size_t(t->size) * elem_bytes(dtype);
  try {
    t->data = dalloc(c, t->bytes);
  } catch (...) {
    delete t;
    throw;
  }
  if (zero) NSG_CUDA(cudaMemsetAsync(t->data, 0, t->bytes, c->stream));
  return t;
}

void free_tensor(nsg_ctx* c, nsg_tensor* t) {
  if (!t) return;
  dfree(c, t->data, t->bytes);
  delete t;
}

double* host_scalars(nsg_ctx* c, size_t n) {
  if (n > c->host_scalars_cap) {
    if (c->host_scalars) cudaFreeHost(c->host_scalars);
    size_t cap = n < 4096 ? 4096 : n;
    NSG_CUDA(cudaMallocHost(&c->host_scalars, cap * sizeof(double)));
    c->host_scalars_cap = cap;
  }
  return c->host_scalars;
}

int* device_flag(nsg_ctx* c) {
  if (!c->dev_flag) {
    NSG_CUDA(cudaMalloc(&c->dev_flag, sizeof(int)));
    NSG_CUDA(cudaMemsetAsync(c->dev_flag, 0, sizeof(int), c->stream));
  }
  c->flag_pending = true;
  return c->dev_flag;
}

void check_device_flag(nsg_ctx* c) {
  if (!c || !c->flag_pending) return;
  c->flag_pending = false;
  int h = 0;
  NSG_CUDA(cudaMemcpyAsync(&h, c->dev_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  if (h) {
    NSG_CUDA(cudaMemsetAsync(c->dev_flag, 0, sizeof(int), c->stream));
    throw Error(NSG_ERR_TIMEOUT, "a tensor-core kernel's bounded mbarrier wait timed out");
  }
}

double* dev_scratch(nsg_ctx* c, size_t n) {
  if (n > c->dev_scratch_cap) {
    if (c->dev_scratch) {
      NSG_CUDA(cudaStreamSynchronize(c->stream));
      NSG_CUDA(cudaFree(c->dev_scratch));
    }
    size_t cap = n < (1 << 16) ? (1 << 16) : n;
    NSG_CUDA(cudaMalloc(&c->dev_scratch, cap * sizeof(double)));
    c->dev_scratch_cap = cap;
  }
  return c->dev_scratch;
}

// Waits for a device flag with the bounded pattern of the library's kernels (poll,
// back off, give up after `polls` polls) and, when the wait runs out, raises the
// context's error flag and returns: the context stays usable.
__global__ void wait_probe_kernel(const int* flag, long long polls, int* err) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const volatile int* f = flag;
  for (long long i = 0; i < polls; ++i) {
    if (*f) return;
    __nanosleep(64);
  }
  atomicExch(err, 1);
}

}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_ctx_set_tuning(nsg_ctx* c, int param, int value) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c, NSG_ERR_INVALID, "null context");
  if (param == NSG_TUNE_SPLITK) {
    NSG_CHECK(value >= 0 && value <= 64, NSG_ERR_INVALID, "tuning: split-K count 0..64");
    c->tune_splitk = value;
  } else if (param == NSG_TUNE_TRIDIAG) {
    NSG_CHECK(value == 0 || value == -1 || value == 2 || value == 4 || value == 8 || value == 16, NSG_ERR_INVALID,
              "tuning: tridiagonalisation path -1, 0, 2, 4, 8 or 16");
    c->tune_tri = value;
  } else if (param == NSG_TUNE_DC_LEAF) {
    NSG_CHECK(value == 0 || (value >= 4 && value <= 32), NSG_ERR_INVALID, "tuning: leaf order 0 or 4..32");
    c->tune_dc_leaf = value;
  } else {
    NSG_CHECK(false, NSG_ERR_INVALID, "tuning: unknown parameter");
  }
  NSG_API_END(c)
}

int nsg_ctx_wait_probe(nsg_ctx* c, int64_t polls) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c, NSG_ERR_INVALID, "null context");
  NSG_CHECK(polls >= 1 && polls <= (int64_t(1) << 24), NSG_ERR_INVALID, "wait probe: polls must be in [1, 2^24]");
  ScopedBuf flag(c, sizeof(int));  // zeroed, and nothing ever sets it
  NSG_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c->stream));
  wait_probe_kernel<<<1, 32, 0, c->stream>>>((const int*)flag.p, (long long)polls, device_flag(c));
  count_launch(c);
  check_launch("wait probe");
  NSG_API_END(c)
}

int nsg_ctx_create(int device, uint64_t hbm_budget_bytes, nsg_ctx** out) {
  nsg_ctx* c = nullptr;
  NSG_API_BEGIN(c)
  NSG_CHECK(out != nullptr, NSG_ERR_INVALID, "out is null");
  int ndev = 0;
  NSG_CUDA(cudaGetDeviceCount(&ndev));
  NSG_CHECK(device >= 0 && device < ndev, NSG_ERR_INVALID, "no such CUDA device");
  NSG_CUDA(cudaSetDevice(device));
  c = new nsg_ctx();
  c->device = device;
  c->budget = hbm_budget_bytes;
  NSG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  cudaMemPool_t pool;
  NSG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
  NSG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  NSG_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  *out = c;
  c = nullptr;
  NSG_API_END(c)
}

static void clear_profile(nsg_ctx* c) {
  for (auto& r : c->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  c->prof.clear();
}

static void clear_phases(nsg_ctx* c) {
  for (auto& r : c->phases) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  c->phases.clear();
  for (auto& e : c->phase_open) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
}

int nsg_ctx_destroy(nsg_ctx* c) {
  if (!c) return NSG_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  clear_profile(c);
  clear_phases(c);
  for (auto& e : c->events)
    if (e) cudaEventDestroy(e);
  if (c->host_scalars) cudaFreeHost(c->host_scalars);
  if (c->dev_scratch) cudaFree(c->dev_scratch);
  if (c->dev_flag) cudaFree(c->dev_flag);
  cudaStreamDestroy(c->stream);
  delete c;
  return NSG_OK;
}

const char* nsg_last_error(const nsg_ctx* c) { return c ? c->err.c_str() : "null context"; }

int nsg_ctx_set_precision(nsg_ctx* c, int precision) {
  NSG_API_BEGIN(c)
  NSG_CHECK(precision >= NSG_PREC_FP64 && precision <= NSG_PREC_OZAKI8, NSG_ERR_INVALID,
            "unknown precision mode");
  c->precision = precision;
  NSG_API_END(c)
}

int nsg_ctx_synchronize(nsg_ctx* c) {
  NSG_API_BEGIN(c)
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  NSG_API_END(c)
}

int nsg_ctx_event_record(nsg_ctx* c, int slot) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && slot >= 0 && slot < 16, NSG_ERR_INVALID, "event slot 0..15");
  if (!c->events[slot]) NSG_CUDA(cudaEventCreate(&c->events[slot]));
  NSG_CUDA(cudaEventRecord(c->events[slot], c->stream));
  NSG_API_END(c)
}

int nsg_ctx_event_elapsed(nsg_ctx* c, int a, int b, float* ms) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && ms && a >= 0 && a < 16 && b >= 0 && b < 16 && c->events[a] && c->events[b], NSG_ERR_INVALID,
            "event slots not recorded");
  NSG_CUDA(cudaEventSynchronize(c->events[b]));
  NSG_CUDA(cudaEventElapsedTime(ms, c->events[a], c->events[b]));
  NSG_API_END(c)
}

int nsg_ctx_profile(nsg_ctx* c, int enable) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c, NSG_ERR_INVALID, "null context");
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  clear_profile(c);
  c->profiling = enable != 0;
  NSG_API_END(c)
}

int nsg_ctx_profile_read(nsg_ctx* c, int cls, uint64_t* launches, double* ms, double* flops) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && cls >= 0 && cls < NSG_PROF_NCLASS, NSG_ERR_INVALID, "profile class out of range");
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  uint64_t n = 0;
  double t = 0, f = 0;
  for (auto& r : c->prof) {
    if (r.cls != cls) continue;
    float e = 0;
    NSG_CUDA(cudaEventElapsedTime(&e, r.a, r.b));
    ++n;
    t += e;
    f += r.flops;
  }
  if (launches) *launches = n;
  if (ms) *ms = t;
  if (flops) *flops = f;
  NSG_API_END(c)
}

int nsg_ctx_timers(nsg_ctx* c, int enable) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c, NSG_ERR_INVALID, "null context");
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  clear_phases(c);
  c->timing = enable != 0;
  NSG_API_END(c)
}

int nsg_ctx_phase(nsg_ctx* c, int phase, int begin) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && phase >= 0 && phase < NSG_PHASE_NCOUNT, NSG_ERR_INVALID, "phase out of range");
  if (c->timing) {
    cudaEvent_t& open = c->phase_open[phase];
    if (begin) {
      NSG_CHECK(open == nullptr, NSG_ERR_INVALID, "phase already open");
      NSG_CUDA(cudaEventCreate(&open));
      NSG_CUDA(cudaEventRecord(open, c->stream));
    } else {
      NSG_CHECK(open != nullptr, NSG_ERR_INVALID, "phase not open");
      cudaEvent_t b = nullptr;
      NSG_CUDA(cudaEventCreate(&b));
      NSG_CUDA(cudaEventRecord(b, c->stream));
      c->phases.push_back({phase, open, b, 0.0});
      open = nullptr;
    }
  }
  NSG_API_END(c)
}

int nsg_get_timers(nsg_ctx* c, uint64_t* counts, double* ms) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && counts && ms, NSG_ERR_INVALID, "null argument");
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  for (int p = 0; p < NSG_PHASE_NCOUNT; ++p) {
    counts[p] = 0;
    ms[p] = 0.0;
  }
  for (auto& r : c->phases) {
    float e = 0;
    NSG_CUDA(cudaEventElapsedTime(&e, r.a, r.b));
    counts[r.cls] += 1;
    ms[r.cls] += e;
  }
  NSG_API_END(c)
}

int nsg_device_memory(int device, uint64_t* free_bytes, uint64_t* total_bytes) {
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return NSG_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return NSG_ERR_CUDA;
  size_t f = 0, t = 0;
  cudaError_t e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return NSG_ERR_CUDA;
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return NSG_OK;
}

int nsg_ctx_memory(const nsg_ctx* c, uint64_t* in_use, uint64_t* peak, uint64_t* budget) {
  if (!c) return NSG_ERR_INVALID;
  if (in_use) *in_use = c->in_use;
  if (peak) *peak = c->peak;
  if (budget) *budget = c->budget;
  return NSG_OK;
}

int nsg_ctx_counters(nsg_ctx* c, uint64_t* out, int reset) {
  if (!c) return NSG_ERR_INVALID;
  if (out) {
    out[0] = c->launches;
    out[1] = c->flops;
    out[2] = c->contractions;
    out[3] = c->applies;
  }
  if (reset) c->launches = c->flops = c->contractions = c->applies = 0;
  return NSG_OK;
}

int nsg_tensor_create(nsg_ctx* c, int dtype, int rank, const int64_t* dims, nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && out, NSG_ERR_INVALID, "null argument");
  *out = new_tensor(c, dtype, rank, dims, true);
  NSG_API_END(c)
}

int nsg_tensor_upload(nsg_ctx* c, int dtype, int rank, const int64_t* dims, const void* host,
                      nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && out && host, NSG_ERR_INVALID, "null argument");
  nsg_tensor* t = new_tensor(c, dtype, rank, dims, false);
  cudaError_t e = cudaMemcpyAsync(t->data, host, t->bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    free_tensor(c, t);
    throw Error(NSG_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
  }
  *out = t;
  NSG_API_END(c)
}

int nsg_tensor_download(nsg_ctx* c, const nsg_tensor* t, void* host) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && t && host, NSG_ERR_INVALID, "null argument");
  NSG_CUDA(cudaMemcpyAsync(host, t->data, t->bytes, cudaMemcpyDeviceToHost, c->stream));
  NSG_CUDA(cudaStreamSynchronize(c->stream));
  NSG_API_END(c)
}

int nsg_tensor_release(nsg_ctx* c, nsg_tensor* t) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c, NSG_ERR_INVALID, "null context");
  free_tensor(c, t);
  NSG_API_END(c)
}

int nsg_tensor_shape(const nsg_tensor* t, int* dtype, int* rank, int64_t* dims) {
  if (!t) return NSG_ERR_INVALID;
  if (dtype) *dtype = t->dtype;
  if (rank) *rank = t->rank;
  if (dims)
    for (int k = 0; k < t->rank; ++k) dims[k] = t->dims[k];
  return NSG_OK;
}

int nsg_tensor_device_ptr(const nsg_tensor* t, void** ptr) {
  if (!t || !ptr) return NSG_ERR_INVALID;
  *ptr = t->data;
  return NSG_OK;
}

int nsg_tensor_copy(nsg_ctx* c, const nsg_tensor* src, nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && src && out, NSG_ERR_INVALID, "null argument");
  nsg_tensor* t = new_tensor(c, src->dtype, src->rank, src->dims, false);
  NSG_CUDA(cudaMemcpyAsync(t->data, src->data, t->bytes, cudaMemcpyDeviceToDevice, c->stream));
  *out = t;
  NSG_API_END(c)
}

int nsg_axpby(nsg_ctx* c, double ar, double ai, const nsg_tensor* x, double br, double bi,
              nsg_tensor* y) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && x && y, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(x->dtype == y->dtype && x->size == y->size, NSG_ERR_INVALID, "axpby: shape/dtype mismatch");
  axpby(c, x->dtype, x->size, ar, ai, x->data, br, bi, y->data);
  NSG_API_END(c)
}

int nsg_dot(nsg_ctx* c, const nsg_tensor* x, const nsg_tensor* y, double* re, double* im) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && x && y, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(x->dtype == y->dtype && x->size == y->size, NSG_ERR_INVALID, "dot: shape/dtype mismatch");
  double out[2] = {0, 0};
  const void* v[1] = {x->data};
  multi_dot(c, x->dtype, x->size, 1, v, y->data, out);
  if (re) *re = out[0];
  if (im) *im = x->dtype == NSG_C128 ? out[1] : 0.0;
  NSG_API_END(c)
}

int nsg_norm(nsg_ctx* c, const nsg_tensor* x, double* out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && x && out, NSG_ERR_INVALID, "null argument");
  *out = norm2(c, x->dtype, x->size, x->data);
  NSG_API_END(c)
}

int nsg_permute(nsg_ctx* c, const nsg_tensor* x, const int* perm, int conj, nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && x && out, NSG_ERR_INVALID, "null argument");
  int64_t dims[NSG_MAX_RANK];
  std::vector<int> seen(x->rank, 0);
  for (int k = 0; k < x->rank; ++k) {
    NSG_CHECK(perm[k] >= 0 && perm[k] < x->rank && !seen[perm[k]], NSG_ERR_INVALID, "bad permutation");
    seen[perm[k]] = 1;
    dims[k] = x->dims[perm[k]];
  }
  nsg_tensor* t = new_tensor(c, x->dtype, x->rank, dims, false);
  permute(c, x, perm, conj != 0, t);
  *out = t;
  NSG_API_END(c)
}

}  // extern "C"
