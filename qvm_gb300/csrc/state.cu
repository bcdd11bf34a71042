// state.cu -- library-wide plumbing and the pure-state lifecycle.
//
// A qvmg_state owns 2^n amplitudes in HBM (double2 or float2, LSB-first
// index) plus small reduction scratch, and its own CUDA stream.  This file
// replaces make-pure-state / allocate-vector / bring-to-zero-state /
// copy-wavefunction of the reference (src/state-representation.lisp:76-152,
// src/allocator.lisp:47-106, src/wavefunction.lisp:80-109).
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <vector>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <mutex>
#include <string>

#include "internal.h"

namespace qvmg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? QVMG_E_NOMEM : QVMG_E_CUDA;
}

static int g_sm_count = 0;
static std::once_flag g_sm_once;

int sm_count() {
  std::call_once(g_sm_once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 1;
  });
  return g_sm_count;
}

int grid_for(uint64_t work, int threads, int per_sm) {
  uint64_t need = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count() * per_sm;
  uint64_t g = std::min<uint64_t>(need, cap);
  return (int)std::max<uint64_t>(g, 1);
}

int check_state(qvmg_state s) {
  if (!s || !s->amps) return fail(QVMG_E_INVALID, "null or freed state handle");
  return QVMG_OK;
}

int check_qubits(qvmg_state s, int k, const int *qubits, int kmax) {
  if (k < 1 || k > kmax)
    return fail(QVMG_E_INVALID, "gate width k=" + std::to_string(k) + " outside 1.." +
                                    std::to_string(kmax));
  if (k > s->nq)
    return fail(QVMG_E_INVALID, "gate on " + std::to_string(k) + " qubits applied to a " +
                                    std::to_string(s->nq) + "-qubit state");
  if (!qubits) return fail(QVMG_E_INVALID, "null qubit tuple");
  for (int i = 0; i < k; ++i) {
    if (qubits[i] < 0 || qubits[i] >= s->nq)
      return fail(QVMG_E_INVALID, "qubit " + std::to_string(qubits[i]) +
                                      " out of range for a " + std::to_string(s->nq) +
                                      "-qubit state");
    for (int j = 0; j < i; ++j)
      if (qubits[j] == qubits[i])
        return fail(QVMG_E_INVALID, "repeated qubit " + std::to_string(qubits[i]));
  }
  return QVMG_OK;
}

// Test hook: the nth device allocation from now fails as out of memory.
static std::atomic<int> g_alloc_fault_countdown{0};

bool alloc_fault_injected() {
  int c = g_alloc_fault_countdown.load();
  while (c > 0) {
    if (g_alloc_fault_countdown.compare_exchange_weak(c, c - 1)) return c == 1;
  }
  return false;
}

int dev_alloc(void **p, size_t bytes, cudaStream_t s) {
  // Keep freed memory in each device's pool: states and plans come and go
  // per request.  The release threshold is a per-pool setting, so it is set
  // once for every device the library allocates on.
  constexpr int kMaxDevices = 64;
  static std::once_flag flags[kMaxDevices];
  static cudaError_t errs[kMaxDevices];
  int dev = 0;
  QVMG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(QVMG_E_INVALID, "device ordinal out of range");
  QVMG_CUDA(once(flags[dev], errs[dev], [dev] {
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, dev);
    uint64_t keep = ~0ull;
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    return e;
  }));
  if (alloc_fault_injected()) {
    *p = nullptr;
    return fail(QVMG_E_NOMEM, "injected device allocation failure (qvmg_debug_fail_alloc)");
  }
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e == cudaErrorMemoryAllocation) {
    // The pool keeps freed blocks; if none is large enough and the device is
    // full, give the unused ones back and retry once.  Only the allocating
    // stream and the library's free stream are waited for (their queued
    // frees land in the pool): a device-wide synchronize would also break
    // a graph capture running on another thread.
    cudaGetLastError();
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess &&
        cudaStreamSynchronize(s) == cudaSuccess &&
        cudaStreamSynchronize(free_stream()) == cudaSuccess &&
        cudaMemPoolTrimTo(pool, 0) == cudaSuccess)
      e = cudaMallocAsync(p, bytes, s);
  }
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return cuda_fail(e, "cudaMallocAsync");
  }
  return QVMG_OK;
}

void dev_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

cudaStream_t free_stream() {
  static std::once_flag flag;
  static cudaStream_t st = nullptr;
  std::call_once(flag, [] { cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking); });
  return st;
}

// Scratch buffers are replaced in the state's stream order: the old one is
// freed after the work already queued that reads it.
int ensure_dvec(qvmg_state s, uint64_t bytes) {
  if (s->dvec_bytes >= bytes) return QVMG_OK;
  dev_free(s->dvec, s->stream);
  s->dvec = nullptr;
  s->dvec_bytes = 0;
  uint64_t want = std::max<uint64_t>(bytes, 1 << 16);
  int rc = dev_alloc((void **)&s->dvec, want, s->stream);
  if (rc) return rc;
  s->dvec_bytes = want;
  return QVMG_OK;
}

int ensure_staging(qvmg_state s, uint64_t bytes) {
  if (s->staging_bytes >= bytes) return QVMG_OK;
  dev_free(s->staging, s->stream);
  s->staging = nullptr;
  s->staging_bytes = 0;
  int rc = dev_alloc(&s->staging, bytes, s->stream);
  if (rc) return rc;
  s->staging_bytes = bytes;
  return QVMG_OK;
}

// Pinned host blocks by power-of-two size class, kept for reuse for the
// life of the process: cudaMallocHost / cudaFreeHost per state stalled the
// serving engine's workers for up to seconds while the GPU was busy.
static std::mutex g_pinned_mu;
static std::map<uint64_t, std::vector<void *>> g_pinned_free;

static uint64_t pinned_class(uint64_t bytes) {
  uint64_t c = 64;
  while (c < bytes) c <<= 1;
  return c;
}

int pinned_get(void **p, uint64_t bytes) {
  const uint64_t c = pinned_class(bytes);
  {
    std::lock_guard<std::mutex> g(g_pinned_mu);
    auto &v = g_pinned_free[c];
    if (!v.empty()) {
      *p = v.back();
      v.pop_back();
      return QVMG_OK;
    }
  }
  cudaError_t e = cudaMallocHost(p, c);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_fail(e, "cudaMallocHost");
  }
  return QVMG_OK;
}

void pinned_put(void *p, uint64_t bytes) {
  if (!p) return;
  std::lock_guard<std::mutex> g(g_pinned_mu);
  g_pinned_free[pinned_class(bytes)].push_back(p);
}

int ensure_pinned(qvmg_state s, uint64_t bytes) {
  if (s->pinned_bytes >= bytes) return QVMG_OK;
  if (s->pinned) {
    QVMG_CUDA(cudaStreamSynchronize(s->stream));  // copies into it are done
    pinned_put(s->pinned, s->pinned_bytes);
    s->pinned = nullptr;
    s->pinned_bytes = 0;
  }
  int rc = pinned_get(&s->pinned, bytes);
  if (rc) return rc;
  s->pinned_bytes = pinned_class(bytes);
  return QVMG_OK;
}

// ---- kernels -------------------------------------------------------------------
__global__ void k_set_amp0(void *amps, int prec) {
  if (prec == QVMG_FP64)
    ((double2 *)amps)[0] = make_double2(1.0, 0.0);
  else
    ((float2 *)amps)[0] = make_float2(1.0f, 0.0f);
}

__global__ void k_f64_to_f32(const double2 *__restrict__ in, float2 *__restrict__ out,
                             uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void k_f32_to_f64(const float2 *__restrict__ in, double2 *__restrict__ out,
                             uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float2 v = in[i];
    out[i] = make_double2((double)v.x, (double)v.y);
  }
}

static int order_after(qvmg_state waiter, qvmg_state producer) {
  if (waiter->stream == producer->stream) return QVMG_OK;
  cudaEvent_t ev;
  QVMG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e1 = cudaEventRecord(ev, producer->stream);
  cudaError_t e2 = cudaStreamWaitEvent(waiter->stream, ev, 0);
  cudaEventDestroy(ev);
  if (e1 != cudaSuccess) return cuda_fail(e1, "cudaEventRecord");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamWaitEvent");
  return QVMG_OK;
}

int order_states(qvmg_state waiter, qvmg_state producer) { return order_after(waiter, producer); }

// Host copy of one chunk from pinned memory, split over a few threads
// (large chunks are bound by a single core's copy rate).
static void parallel_copy(void *dst, const void *src, size_t bytes) {
  const size_t kMinPerThread = 4u << 20;
  int nt = (int)std::min<size_t>(8, bytes / kMinPerThread);
  if (nt <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> th;
  const size_t part = (bytes / nt + 63) & ~(size_t)63;
  for (int i = 0; i < nt; ++i) {
    const size_t b0 = (size_t)i * part;
    if (b0 >= bytes) break;
    const size_t len = std::min(part, bytes - b0);
    th.emplace_back([=] { std::memcpy((char *)dst + b0, (const char *)src + b0, len); });
  }
  for (auto &t : th) t.join();
}

int stream_to_host(qvmg_state s, uint64_t count, size_t elem, void *out, ProduceFn produce,
                   void *ctx) {
  const uint64_t chunk = std::min<uint64_t>(count, (64ull << 20) / elem);
  const size_t cb = (size_t)chunk * elem;
  int rc;
  if (produce && (rc = ensure_staging(s, 2 * cb))) return rc;
  if ((rc = ensure_pinned(s, 2 * cb))) return rc;
  for (auto &e : s->xfer_ev)
    if (!e) QVMG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  const uint64_t nchunks = (count + chunk - 1) / chunk;
  for (uint64_t i = 0; i <= nchunks; ++i) {
    if (i < nchunks) {
      const int b = (int)(i & 1);
      const uint64_t off = i * chunk, n = std::min(chunk, count - off);
      const void *src;
      if (produce) {
        void *dst = (char *)s->staging + b * cb;
        if ((rc = produce(s, off, n, dst, ctx))) return rc;
        src = dst;
      } else {
        src = (const char *)s->amps + off * elem;
      }
      QVMG_CUDA(cudaMemcpyAsync((char *)s->pinned + b * cb, src, n * elem, cudaMemcpyDeviceToHost,
                                s->stream));
      QVMG_CUDA(cudaEventRecord(s->xfer_ev[b], s->stream));
    }
    if (i >= 1) {
      const uint64_t j = i - 1;
      const int b = (int)(j & 1);
      const uint64_t off = j * chunk, n = std::min(chunk, count - off);
      QVMG_CUDA(cudaEventSynchronize(s->xfer_ev[b]));
      parallel_copy((char *)out + off * elem, (const char *)s->pinned + b * cb, n * elem);
    }
  }
  return QVMG_OK;
}

static int produce_f64_from_f32(qvmg_state s, uint64_t off, uint64_t n, void *dst, void *) {
  k_f32_to_f64<<<grid_for(n, 256), 256, 0, s->stream>>>((const float2 *)s->amps + off,
                                                        (double2 *)dst, n);
  QVMG_CHECK_LAUNCH("k_f32_to_f64");
  return QVMG_OK;
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

const char *qvmg_last_error(void) { return g_last_error.c_str(); }

int qvmg_abi_version(void) { return QVMG_ABI_VERSION; }

int qvmg_debug_fail_alloc(int nth) {
  if (nth < 0) return fail(QVMG_E_INVALID, "negative allocation countdown");
  g_alloc_fault_countdown.store(nth);
  return QVMG_OK;
}

int qvmg_device_info(int *sms, uint64_t *free_bytes, uint64_t *total_bytes) {
  size_t f = 0, t = 0;
  QVMG_CUDA(cudaMemGetInfo(&f, &t));
  if (sms) *sms = sm_count();
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return QVMG_OK;
}

uint64_t qvmg_state_bytes(int nqubits, int precision) {
  if (nqubits < 1 || nqubits > QVMG_MAX_QUBITS) return 0;
  if (precision != QVMG_FP64 && precision != QVMG_FP32) return 0;
  uint64_t len = 1ull << nqubits;
  uint64_t nblocks = nqubits > kSampleBlockBits ? (len >> kSampleBlockBits) : 1;
  return len * amp_bytes(precision) + (nblocks + 1) * sizeof(double) +
         2 * kReduceBlocks * sizeof(double) + sizeof(MeasResult);
}

int qvmg_state_create(int nqubits, int precision, qvmg_state *out) {
  if (!out) return fail(QVMG_E_INVALID, "null output handle");
  *out = nullptr;
  if (nqubits < 1 || nqubits > QVMG_MAX_QUBITS)
    return fail(QVMG_E_INVALID, "qubit count " + std::to_string(nqubits) + " outside 1.." +
                                    std::to_string(QVMG_MAX_QUBITS));
  if (precision != QVMG_FP64 && precision != QVMG_FP32)
    return fail(QVMG_E_INVALID, "precision must be QVMG_FP64 or QVMG_FP32");
  qvmg_state s = new qvmg_state_s();
  s->nq = nqubits;
  s->prec = precision;
  s->len = 1ull << nqubits;
  s->nblocks = nqubits > kSampleBlockBits ? (s->len >> kSampleBlockBits) : 1;
  cudaGetDevice(&s->device);
  int rc = QVMG_OK;
  cudaError_t e;
  do {
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
      rc = cuda_fail(e, "cudaStreamCreate");
      break;
    }
    if ((rc = dev_alloc(&s->amps, s->len * amp_bytes(precision), s->stream))) break;
    if ((rc = dev_alloc((void **)&s->partials, 2 * kReduceBlocks * sizeof(double), s->stream)))
      break;
    if ((rc = dev_alloc((void **)&s->block_sums, (s->nblocks + 1) * sizeof(double), s->stream)))
      break;
    if ((rc = dev_alloc((void **)&s->dres, sizeof(MeasResult), s->stream))) break;
    // pooled memory is not zeroed: the status word must start at 0
    if ((e = cudaMemsetAsync(s->dres, 0, sizeof(MeasResult), s->stream)) != cudaSuccess) {
      rc = cuda_fail(e, "cudaMemsetAsync(result)");
      break;
    }
    if ((rc = pinned_get((void **)&s->hres, sizeof(MeasResult)))) break;
  } while (0);
  if (rc == QVMG_OK) rc = qvmg_state_reset(s);
  if (rc != QVMG_OK) {
    std::string msg = g_last_error;
    qvmg_state_free(s);
    g_last_error = msg;
    return rc;
  }
  *out = s;
  return QVMG_OK;
}

int qvmg_state_free(qvmg_state s) {
  if (!s) return QVMG_OK;
  // device memory goes back to the pool in this stream's order (work of other
  // states that read it is ordered into this stream by the cross-state calls);
  // the pinned host buffers wait for this stream only
  if (s->stream) {
    dev_free(s->amps, s->stream);
    dev_free(s->partials, s->stream);
    dev_free(s->block_sums, s->stream);
    dev_free(s->dres, s->stream);
    dev_free(s->staging, s->stream);
    dev_free(s->dvec, s->stream);
    cudaStreamSynchronize(s->stream);
  }
  pinned_put(s->hres, sizeof(MeasResult));
  pinned_put(s->pinned, s->pinned_bytes);
  for (auto &e : s->xfer_ev)
    if (e) cudaEventDestroy(e);
  if (s->stream) cudaStreamDestroy(s->stream);
  s->amps = nullptr;
  delete s;
  return QVMG_OK;
}

int qvmg_device_reserve(uint64_t bytes) {
  // in blocks of up to 16 GiB (a 30-qubit FP64 state), allocated together and
  // then freed into the pool, which keeps them
  const uint64_t block = 16ull << 30;
  cudaStream_t st = free_stream();
  std::vector<void *> got;
  int rc = QVMG_OK;
  for (uint64_t done = 0; done < bytes && rc == QVMG_OK;) {
    const uint64_t b = std::min(block, bytes - done);
    void *p = nullptr;
    rc = dev_alloc(&p, b, st);
    if (rc == QVMG_OK) {
      got.push_back(p);
      done += b;
    }
  }
  for (void *p : got) dev_free(p, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (rc) {
    // a failed reservation keeps nothing: the pool's unused memory goes back
    // to the device, so that other allocators in the process still find it
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
      cudaMemPoolTrimTo(pool, 0);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  return QVMG_OK;
}

int qvmg_state_set_priority(qvmg_state s, int priority) {
  int rc = check_state(s);
  if (rc) return rc;
  if (priority < -1 || priority > 1) return fail(QVMG_E_INVALID, "priority must be -1, 0 or 1");
  int least = 0, greatest = 0;
  QVMG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  const int want = priority == 1 ? greatest : least;
  const int have = s->priority == 1 ? greatest : least;
  if (want != have) {
    // buffers were allocated in the old stream's order: finish it first
    QVMG_CUDA(cudaStreamSynchronize(s->stream));
    cudaStream_t ns = nullptr;
    QVMG_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, want));
    cudaStreamDestroy(s->stream);
    s->stream = ns;
  }
  s->priority = priority;
  return QVMG_OK;
}

int qvmg_state_info(qvmg_state s, int *nqubits, int *precision) {
  int rc = check_state(s);
  if (rc) return rc;
  if (nqubits) *nqubits = s->nq;
  if (precision) *precision = s->prec;
  return QVMG_OK;
}

int qvmg_state_reset(qvmg_state s) {
  int rc = check_state(s);
  if (rc) return rc;
  QVMG_CUDA(cudaMemsetAsync(s->amps, 0, s->len * amp_bytes(s->prec), s->stream));
  k_set_amp0<<<1, 1, 0, s->stream>>>(s->amps, s->prec);
  QVMG_CHECK_LAUNCH("k_set_amp0");
  return QVMG_OK;
}

// Chunk size for precision-converting transfers (in amplitudes).
static const uint64_t kChunk = 1ull << 22;

int qvmg_state_upload(qvmg_state s, const double *amps) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!amps) return fail(QVMG_E_INVALID, "null host buffer");
  if (s->prec == QVMG_FP64) {
    QVMG_CUDA(cudaMemcpyAsync(s->amps, amps, s->len * 16, cudaMemcpyHostToDevice, s->stream));
    QVMG_CUDA(cudaStreamSynchronize(s->stream));
    return QVMG_OK;
  }
  uint64_t chunk = std::min(kChunk, s->len);
  if ((rc = ensure_staging(s, chunk * 16))) return rc;
  for (uint64_t off = 0; off < s->len; off += chunk) {
    uint64_t n = std::min(chunk, s->len - off);
    QVMG_CUDA(cudaMemcpyAsync(s->staging, amps + 2 * off, n * 16, cudaMemcpyHostToDevice,
                              s->stream));
    k_f64_to_f32<<<grid_for(n, 256), 256, 0, s->stream>>>((const double2 *)s->staging,
                                                          (float2 *)s->amps + off, n);
    QVMG_CHECK_LAUNCH("k_f64_to_f32");
  }
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

int qvmg_state_download(qvmg_state s, double *amps) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!amps) return fail(QVMG_E_INVALID, "null host buffer");
  return stream_to_host(s, s->len, 16, amps,
                        s->prec == QVMG_FP64 ? nullptr : produce_f64_from_f32, nullptr);
}

int qvmg_state_copy(qvmg_state dst, qvmg_state src) {
  int rc = check_state(dst);
  if (rc) return rc;
  if ((rc = check_state(src))) return rc;
  if (dst->nq != src->nq)
    return fail(QVMG_E_INVALID, "copy between states of different qubit counts");
  if (dst == src) return QVMG_OK;
  if ((rc = order_after(dst, src))) return rc;
  if (dst->prec == src->prec) {
    QVMG_CUDA(cudaMemcpyAsync(dst->amps, src->amps, dst->len * amp_bytes(dst->prec),
                              cudaMemcpyDeviceToDevice, dst->stream));
  } else if (src->prec == QVMG_FP64) {
    k_f64_to_f32<<<grid_for(dst->len, 256), 256, 0, dst->stream>>>(
        (const double2 *)src->amps, (float2 *)dst->amps, dst->len);
    QVMG_CHECK_LAUNCH("k_f64_to_f32");
  } else {
    k_f32_to_f64<<<grid_for(dst->len, 256), 256, 0, dst->stream>>>(
        (const float2 *)src->amps, (double2 *)dst->amps, dst->len);
    QVMG_CHECK_LAUNCH("k_f32_to_f64");
  }
  // The source must not be modified before the copy has read it.
  return order_after(src, dst);
}

int qvmg_state_sync(qvmg_state s) {
  int rc = check_state(s);
  if (rc) return rc;
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

}  // extern "C"
