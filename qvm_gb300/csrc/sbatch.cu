// sbatch.cu -- many small, uneven programs in one persistent launch.
//
// The reference runs one QVM per request and re-runs a program per trial
// (app/src/api/multishot.lisp:87-101); its small programs pay the whole
// per-request path each time.  Here a batch of programs -- each its own
// qubit count (<= 13 in FP32, <= 12 in FP64), gate list and shot count --
// runs in one persistent kernel: each CTA takes the next program from a
// device work queue (an atomic counter, largest states first), keeps the
// state in shared memory from |0...0> to the last gate, applies every gate
// as a dense k-qubit block (k <= 3; the gather -> matvec -> scatter of
// apply-matrix-operator, src/wavefunction.lisp:308-330, in the state's own
// precision), writes the final state to the batch's slab and samples its
// shots from the CDF (smallest i with C(i) >= draw,
// src/measurement.lisp:246-288; FP32 states sample the renormalised
// distribution, as qvmg_sample does).  The queue reset and the kernel are
// one captured CUDA graph, replayed on every run with the same shot counts.
// A program is processed by one CTA whatever else is in the batch, so its
// results do not depend on the batch it runs in.  Spin-free: no CTA waits
// on another.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

constexpr int kSbThreads = 256;
constexpr int kSbMaxK = 3;
constexpr int kSbSubBits = 7;           // 128-amplitude CDF sub-blocks
constexpr int kSbStateBytes = 1 << 16;  // 2^13 FP32 or 2^12 FP64 amplitudes

struct SbJob {
  unsigned long long op_off;     // first op of the program
  unsigned long long shot_off;   // first draw / shot of the program
  unsigned long long state_off;  // amplitude offset in the state slab
  int n, nops, nshots, id;
};

struct SbOp {
  int k;
  int q[kSbMaxK];                // nat-tuple order: q[0] is the matrix LSB
  unsigned long long m_off;      // complex offset of the 2^k x 2^k matrix
};

struct SbArgs {
  int njobs;
  int pad;
  const SbJob *jobs;
  const SbOp *ops;
  const void *mats;              // complex, the batch's precision
  void *states;
  const double *draws;
  unsigned long long *shots;
  unsigned int *counter;
};

__device__ __forceinline__ unsigned sb_inject0(unsigned x, int q) {
  return ((x >> q) << (q + 1)) | (x & ((1u << q) - 1u));
}

template <typename T, int K>
__device__ __forceinline__ void sb_dense(typename CT<T>::C *st, int n, const SbOp &op,
                                         const typename CT<T>::C *m) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.q[i];
#pragma unroll
  for (int i = 1; i < K; ++i)
#pragma unroll
    for (int j = i; j > 0; --j)
      if (sp[j - 1] > sp[j]) {
        const int x = sp[j];
        sp[j] = sp[j - 1];
        sp[j - 1] = x;
      }
  unsigned off[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    unsigned o = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1u << op.q[j];
    off[c] = o;
  }
  const unsigned ngroups = 1u << (n - K);
  for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x) {
    unsigned b = g;
#pragma unroll
    for (int s = 0; s < K; ++s) b = sb_inject0(b, sp[s]);
    C v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = st[b | off[c]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      C acc = CT<T>::make(0, 0);
#pragma unroll
      for (int c = 0; c < D; ++c) cmac(acc, m[r * D + c], v[c]);
      st[b | off[r]] = acc;
    }
  }
}

__device__ __forceinline__ double sb_prob(float2 v) { return prob_f64(v); }
__device__ __forceinline__ double sb_prob(double2 v) { return prob_f64(v); }

template <typename T>
__global__ void __launch_bounds__(kSbThreads) k_small_batch(const __grid_constant__ SbArgs A) {
  using C = typename CT<T>::C;
  extern __shared__ __align__(16) unsigned char smem[];
  C *st = reinterpret_cast<C *>(smem);
  C *mat = reinterpret_cast<C *>(smem + kSbStateBytes);        // 64 entries
  double *sub = reinterpret_cast<double *>(mat + 64);          // 64 sub-block prefixes
  __shared__ int s_job;
  const C *mats = reinterpret_cast<const C *>(A.mats);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_job = (int)atomicAdd(A.counter, 1u);
    __syncthreads();
    const int jn = s_job;
    if (jn >= A.njobs) break;
    const SbJob J = A.jobs[jn];
    const unsigned len = 1u << J.n;
    for (unsigned x = threadIdx.x; x < len; x += blockDim.x)
      st[x] = x == 0 ? CT<T>::make(1, 0) : CT<T>::make(0, 0);
    for (int o = 0; o < J.nops; ++o) {
      const SbOp op = A.ops[J.op_off + o];
      const int d = 1 << op.k;
      __syncthreads();  // the previous op is done with the state and `mat`
      for (int i = threadIdx.x; i < d * d; i += blockDim.x) mat[i] = mats[op.m_off + i];
      __syncthreads();
      if (op.k == 1) sb_dense<T, 1>(st, J.n, op, mat);
      else if (op.k == 2) sb_dense<T, 2>(st, J.n, op, mat);
      else sb_dense<T, 3>(st, J.n, op, mat);
    }
    __syncthreads();
    C *psi = reinterpret_cast<C *>(A.states) + J.state_off;
    for (unsigned x = threadIdx.x; x < len; x += blockDim.x) psi[x] = st[x];
    // CDF: sums of 128-amplitude sub-blocks (one warp each), then their
    // inclusive prefix by warp 0
    const int sbits = J.n < kSbSubBits ? J.n : kSbSubBits;
    const unsigned nsub = len >> sbits;
    for (unsigned sb = warp; sb < nsub; sb += nwarps) {
      double acc = 0.0;
      for (unsigned j = lane; j < (1u << sbits); j += 32) acc += sb_prob(st[(sb << sbits) + j]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) sub[sb] = acc;
    }
    __syncthreads();
    if (warp == 0) {
      double run = 0.0;
      for (unsigned base = 0; base < nsub; base += 32) {
        double v = base + lane < nsub ? sub[base + lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const double y = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += y;
        }
        if (base + lane < nsub) sub[base + lane] = run + v;
        run += __shfl_sync(0xffffffffu, v, 31);
      }
    }
    __syncthreads();
    // shots: one warp per draw
    for (int t = warp; t < J.nshots; t += nwarps) {
      const double draw = A.draws[J.shot_off + t];
      const double p = sizeof(typename CT<T>::C) == 8 ? draw * sub[nsub - 1] : draw;
      unsigned lo = 0, hi = nsub;  // first sub-block whose prefix reaches p
      while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (sub[mid] >= p) hi = mid;
        else lo = mid + 1;
      }
      unsigned long long res = len - 1;
      if (lo < nsub) {
        double run = lo ? sub[lo - 1] : 0.0;
        res = ((unsigned long long)(lo + 1) << sbits) - 1;
        for (unsigned c0 = 0; c0 < (1u << sbits); c0 += 32) {
          const bool valid = c0 + lane < (1u << sbits);
          const double pr = valid ? sb_prob(st[(lo << sbits) + c0 + lane]) : 0.0;
          double sc = pr;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, sc, o);
            if (lane >= o) sc += y;
          }
          const unsigned msk = __ballot_sync(0xffffffffu, valid && run + sc >= p);
          if (msk) {
            res = ((unsigned long long)lo << sbits) + c0 + (__ffs(msk) - 1);
            break;
          }
          run += __shfl_sync(0xffffffffu, sc, 31);
        }
      }
      if (lane == 0) A.shots[J.shot_off + t] = res;
    }
  }
}

constexpr int kSbSmemBytes = kSbStateBytes + 64 * 16 + 64 * 8;

}  // namespace qvmg

struct qvmg_sbatch_s {
  int njobs = 0, prec = QVMG_FP64;
  std::vector<int> n, nshots;
  std::vector<unsigned long long> state_off, shot_off;
  unsigned long long total_shots = 0;
  qvmg::SbArgs args{};
  void *dbuf = nullptr;   // jobs, ops, matrices
  void *states = nullptr;
  double *draws = nullptr;
  unsigned long long *shots = nullptr;
  unsigned int *counter = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  uint64_t bytes = 0;
};

using namespace qvmg;

static void sbatch_release(qvmg_sbatch b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->dbuf);
  cudaFree(b->states);
  cudaFree(b->draws);
  cudaFree(b->shots);
  cudaFree(b->counter);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" {

int qvmg_sbatch_create(int precision, int njobs, const int *nqubits, const int *nops,
                       const int *op_k, const int *op_qubits, const double *matrices,
                       const int *nshots, qvmg_sbatch *out) {
  if (!out) return fail(QVMG_E_INVALID, "null output handle");
  *out = nullptr;
  if (precision != QVMG_FP64 && precision != QVMG_FP32)
    return fail(QVMG_E_INVALID, "precision must be QVMG_FP64 or QVMG_FP32");
  if (njobs < 1 || !nqubits || !nops || !nshots)
    return fail(QVMG_E_INVALID, "empty batch or null array");
  const int nmax = precision == QVMG_FP32 ? 13 : 12;
  const size_t csz = precision == QVMG_FP32 ? 8 : 16;
  std::vector<SbJob> jobs(njobs);
  std::vector<SbOp> ops;
  std::vector<double> mats;  // interleaved (re, im), converted below
  size_t ooff = 0, qoff = 0, moff = 0;
  unsigned long long shot_total = 0;
  for (int i = 0; i < njobs; ++i) {
    const int n = nqubits[i];
    if (n < 1 || n > nmax)
      return fail(QVMG_E_INVALID, "program " + std::to_string(i) + ": " + std::to_string(n) +
                                      " qubits outside 1.." + std::to_string(nmax) +
                                      " for this precision");
    if (nops[i] < 0) return fail(QVMG_E_INVALID, "negative op count");
    if (nshots[i] < 0) return fail(QVMG_E_INVALID, "negative shot count");
    if (nops[i] > 0 && (!op_k || !op_qubits || !matrices))
      return fail(QVMG_E_INVALID, "ops given without their arrays");
    SbJob &J = jobs[i];
    J.n = n;
    J.nops = nops[i];
    J.nshots = nshots[i];
    J.id = i;
    J.op_off = ops.size();
    J.shot_off = shot_total;
    shot_total += (unsigned long long)nshots[i];
    for (int o = 0; o < nops[i]; ++o, ++ooff) {
      SbOp op{};
      op.k = op_k[ooff];
      if (op.k < 1 || op.k > kSbMaxK || op.k > n)
        return fail(QVMG_E_INVALID, "program " + std::to_string(i) + ": gate width " +
                                        std::to_string(op.k) + " outside 1..3 or above n");
      for (int j = 0; j < op.k; ++j) {
        const int q = op_qubits[qoff + j];
        if (q < 0 || q >= n)
          return fail(QVMG_E_INVALID, "program " + std::to_string(i) + ": qubit " +
                                          std::to_string(q) + " out of range");
        for (int l = 0; l < j; ++l)
          if (op.q[l] == q)
            return fail(QVMG_E_INVALID, "program " + std::to_string(i) + ": repeated qubit");
        op.q[j] = q;
      }
      qoff += op.k;
      const size_t d = (size_t)1 << op.k;
      op.m_off = mats.size() / 2;
      mats.insert(mats.end(), matrices + 2 * moff, matrices + 2 * (moff + d * d));
      moff += d * d;
      ops.push_back(op);
    }
  }
  // largest states first: the queue hands them out before the small ones
  std::vector<int> order(njobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return jobs[a].n > jobs[c].n; });
  qvmg_sbatch b = new qvmg_sbatch_s();
  b->njobs = njobs;
  b->prec = precision;
  b->n.assign(nqubits, nqubits + njobs);
  b->nshots.assign(nshots, nshots + njobs);
  b->state_off.assign(njobs, 0);
  b->shot_off.assign(njobs, 0);
  b->total_shots = shot_total;
  std::vector<SbJob> sorted(njobs);
  unsigned long long soff = 0;
  for (int r = 0; r < njobs; ++r) {
    SbJob J = jobs[order[r]];
    J.state_off = soff;
    b->state_off[J.id] = soff;
    b->shot_off[J.id] = J.shot_off;
    soff += 1ull << J.n;
    sorted[r] = J;
  }
  std::vector<unsigned char> host;
  auto put = [&](const void *p, size_t bytes) {
    size_t at = (host.size() + 15) & ~(size_t)15;
    host.resize(at + bytes);
    if (bytes) std::memcpy(host.data() + at, p, bytes);
    return at;
  };
  const size_t jb = put(sorted.data(), sorted.size() * sizeof(SbJob));
  const size_t ob = put(ops.data(), ops.size() * sizeof(SbOp));
  size_t mb;
  if (precision == QVMG_FP64) {
    mb = put(mats.data(), mats.size() * sizeof(double));
  } else {
    std::vector<float> f(mats.begin(), mats.end());
    mb = put(f.data(), f.size() * sizeof(float));
  }
  host.resize(host.size() + 16);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
#define SBCHK(call, what)                          \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) {                       \
      sbatch_release(b);                           \
      return cuda_fail(_e, what);                  \
    }                                              \
  } while (0)
  SBCHK(e, "cudaStreamCreate");
  SBCHK(cudaMalloc(&b->dbuf, host.size()), "cudaMalloc(batch programs)");
  SBCHK(cudaMemcpyAsync(b->dbuf, host.data(), host.size(), cudaMemcpyHostToDevice, b->stream),
        "cudaMemcpyAsync(batch programs)");
  SBCHK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
  SBCHK(cudaMalloc(&b->states, soff * csz), "cudaMalloc(batch states)");
  SBCHK(cudaMalloc(&b->draws, sizeof(double) * std::max<unsigned long long>(shot_total, 1)),
        "cudaMalloc(batch draws)");
  SBCHK(cudaMalloc(&b->shots, sizeof(unsigned long long) * std::max<unsigned long long>(shot_total, 1)),
        "cudaMalloc(batch shots)");
  SBCHK(cudaMalloc(&b->counter, sizeof(unsigned int)), "cudaMalloc(counter)");
#undef SBCHK
  b->bytes = host.size() + soff * csz + shot_total * 16 + 4;
  SbArgs &A = b->args;
  A.njobs = njobs;
  A.jobs = (const SbJob *)((unsigned char *)b->dbuf + jb);
  A.ops = (const SbOp *)((unsigned char *)b->dbuf + ob);
  A.mats = (const void *)((unsigned char *)b->dbuf + mb);
  A.states = b->states;
  A.draws = b->draws;
  A.shots = b->shots;
  A.counter = b->counter;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  e = once(attr_once, attr_err, [] {
    cudaError_t r = cudaFuncSetAttribute(k_small_batch<float>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSbSmemBytes);
    if (r == cudaSuccess)
      r = cudaFuncSetAttribute(k_small_batch<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kSbSmemBytes);
    return r;
  });
  if (e != cudaSuccess) {
    sbatch_release(b);
    return cuda_fail(e, "cudaFuncSetAttribute(k_small_batch)");
  }
  *out = b;
  return QVMG_OK;
}

int qvmg_sbatch_run(qvmg_sbatch b, const double *draws, uint64_t *shots) {
  if (!b) return fail(QVMG_E_INVALID, "null batch");
  if (b->total_shots > 0 && (!draws || !shots))
    return fail(QVMG_E_INVALID, "the batch has shots: draws and output are required");
  for (unsigned long long i = 0; draws && i < b->total_shots; ++i)
    if (!(draws[i] >= 0.0 && draws[i] <= 1.0))
      return fail(QVMG_E_INVALID, "draws must lie in [0, 1]");
  if (b->total_shots > 0)
    QVMG_CUDA(cudaMemcpyAsync(b->draws, draws, sizeof(double) * b->total_shots,
                              cudaMemcpyHostToDevice, b->stream));
  if (!b->graph) {
    // the queue reset and the persistent kernel as one graph, replayed per run
    cudaGraph_t g;
    QVMG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->counter, 0, sizeof(unsigned int), b->stream);
    const int grid = std::min(b->njobs, sm_count() * 3);
    if (b->prec == QVMG_FP32)
      k_small_batch<float><<<grid, kSbThreads, kSbSmemBytes, b->stream>>>(b->args);
    else
      k_small_batch<double><<<grid, kSbThreads, kSbSmemBytes, b->stream>>>(b->args);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) return cuda_fail(le, "k_small_batch launch");
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      b->graph = nullptr;
      return cuda_fail(ie, "cudaGraphInstantiate");
    }
  }
  QVMG_CUDA(cudaGraphLaunch(b->graph, b->stream));
  if (b->total_shots > 0)
    QVMG_CUDA(cudaMemcpyAsync(shots, b->shots, sizeof(unsigned long long) * b->total_shots,
                              cudaMemcpyDeviceToHost, b->stream));
  QVMG_CUDA(cudaStreamSynchronize(b->stream));
  return QVMG_OK;
}

int qvmg_sbatch_shot_offset(qvmg_sbatch b, int program, uint64_t *offset) {
  if (!b || !offset) return fail(QVMG_E_INVALID, "null batch or output");
  if (program < 0 || program >= b->njobs) return fail(QVMG_E_INVALID, "program out of range");
  *offset = b->shot_off[program];
  return QVMG_OK;
}

int qvmg_sbatch_state(qvmg_sbatch b, int program, double *amps) {
  if (!b || !amps) return fail(QVMG_E_INVALID, "null batch or buffer");
  if (program < 0 || program >= b->njobs) return fail(QVMG_E_INVALID, "program out of range");
  const uint64_t len = 1ull << b->n[program];
  if (b->prec == QVMG_FP64) {
    QVMG_CUDA(cudaMemcpyAsync(amps, (double2 *)b->states + b->state_off[program],
                              len * sizeof(double2), cudaMemcpyDeviceToHost, b->stream));
    QVMG_CUDA(cudaStreamSynchronize(b->stream));
    return QVMG_OK;
  }
  std::vector<float2> tmp(len);
  QVMG_CUDA(cudaMemcpyAsync(tmp.data(), (float2 *)b->states + b->state_off[program],
                            len * sizeof(float2), cudaMemcpyDeviceToHost, b->stream));
  QVMG_CUDA(cudaStreamSynchronize(b->stream));
  for (uint64_t i = 0; i < len; ++i) {
    amps[2 * i] = tmp[i].x;
    amps[2 * i + 1] = tmp[i].y;
  }
  return QVMG_OK;
}

uint64_t qvmg_sbatch_bytes(qvmg_sbatch b) { return b ? b->bytes : 0; }

int qvmg_sbatch_free(qvmg_sbatch b) {
  sbatch_release(b);
  return QVMG_OK;
}

}  // extern "C"
