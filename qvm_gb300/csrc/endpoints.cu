// endpoints.cu -- the server endpoints' device work on a resident state.
//
// The reference's multishot-measure endpoint reloads a copy of the prepared
// state and measures the requested qubits once per trial
// (app/src/api/multishot-measure.lisp:12-35,93-109); its multishot endpoint
// re-runs the whole program per trial (app/src/api/multishot.lisp:87-101).
// When the measurements are the last thing a program does, every trial sees
// the same pre-measurement state, so a trial's outcome depends only on the
// marginal distribution of the measured qubits.  Here that marginal is
// reduced once on the device (one read of the state), and the trials are
// replayed on the host from it: the same per-qubit probabilities, the same
// draw per measurement, the same skip of the draw when p1 = 0
// (src/measurement.lisp:87-105) or the compiled rule (bit 0 iff draw < p0,
// src/compile-gate.lisp:221-254).
//
// The wavefunction and probabilities endpoints stream amplitudes as
// big-endian IEEE doubles (app/src/handle-request.lisp:132-175,
// app/src/utilities.lisp:40-87); the byte swap runs on the device and the
// host receives the wire bytes directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

// ---- marginal probabilities ---------------------------------------------------
//
// out[m] = sum of |a_i|^2 over the i whose bits at qubits[0..k-1] spell m
// (bit j of m <-> qubits[j]).  Deterministic: a fixed partition of the
// state, per-warp shared-memory histograms written by one warp each in a
// fixed order, and a fixed-order sum of the per-CTA partial histograms.
//
// The measured qubits, sorted by position, split into "local" ones (the
// lowest min(k, 10)) whose bins a CTA keeps in shared memory, and "group"
// ones (the rest, positions >= 10): each group of CTAs handles the
// amplitudes with one fixed value of the group bits, so a CTA never holds
// more than 2^10 bins.  Within a warp, 32 consecutive amplitudes differ only
// in bits 0..4: a lane sums its own amplitudes while the warp-uniform bins
// stay the same, and on a change the warp folds the unmeasured lane bits
// with shuffles (a fixed butterfly) before one lane per bin adds the sum.
constexpr int kMarginalMaxQubits = 20;
constexpr int kMarginalLocalMax = 10;
constexpr int kMarginalThreads = 256;
constexpr int kMarginalWarps = kMarginalThreads / 32;
constexpr int kMarginalCtas = 1024;  // target CTAs per call (fixed: deterministic)

struct MarginalArgs {
  int kh;                 // group bits
  int nl;                 // local bits
  int C;                  // CTAs per group
  int pad;
  int gpos[kMarginalMaxQubits];  // group positions, ascending
  int lpos[kMarginalLocalMax];   // local positions, ascending
  unsigned long long count;      // amplitudes per group
  unsigned long long R;          // amplitudes per CTA
  unsigned long long wlen;       // amplitudes per warp (multiple of 32)
};

__device__ __forceinline__ double prob64(double2 v) { return fma(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ double prob64(float2 v) {
  const double x = v.x, y = v.y;  // exact squares in FP64
  return fma(x, x, y * y);
}

template <typename C>
__global__ void __launch_bounds__(kMarginalThreads)
    k_marginal(const C *__restrict__ a, const __grid_constant__ MarginalArgs p,
               double *__restrict__ partial) {
  extern __shared__ double hist[];  // kMarginalWarps x 2^nl
  const int nb = 1 << p.nl;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kMarginalWarps * nb; i += kMarginalThreads) hist[i] = 0.0;
  __syncthreads();
  const unsigned g = blockIdx.x / p.C, c = blockIdx.x % p.C;
  unsigned lane_meas = 0;
  int lane_part = 0;
  for (int r = 0; r < p.nl; ++r)
    if (p.lpos[r] < 5) {
      lane_meas |= 1u << p.lpos[r];
      lane_part |= ((lane >> p.lpos[r]) & 1) << r;
    }
  const unsigned lane_free = 31u & ~lane_meas;  // warp-uniform
  const bool leader = (lane & lane_free) == 0;
  double *h = hist + w * nb;
  const unsigned long long cstart = (unsigned long long)c * p.R;
  const unsigned long long cend = min(cstart + p.R, p.count);
  const unsigned long long wstart = cstart + (unsigned long long)w * p.wlen;
  const unsigned long long wend = min(wstart + p.wlen, cend);
  double acc = 0.0;
  int cur = -1;  // warp-uniform bins of the running sums
  auto flush = [&]() {
#pragma unroll
    for (int b = 0; b < 5; ++b)
      if ((lane_free >> b) & 1u) acc += __shfl_xor_sync(0xffffffffu, acc, 1 << b);
    if (leader) h[cur | lane_part] += acc;
    acc = 0.0;
  };
  for (unsigned long long j0 = wstart; j0 < wend; j0 += 32) {
    // expand the group-compressed index: insert the group bits (all >= 10,
    // so bits 0..4 stay the lane's)
    unsigned long long i0 = j0;
    for (int r = 0; r < p.kh; ++r) {
      const int q = p.gpos[r];
      const unsigned long long lo = i0 & ((1ull << q) - 1ull);
      i0 = ((((i0 >> q) << 1) | ((g >> r) & 1u)) << q) | lo;
    }
    int mid = 0;
    for (int r = 0; r < p.nl; ++r)
      if (p.lpos[r] >= 5) mid |= (int)((i0 >> p.lpos[r]) & 1ull) << r;
    if (mid != cur) {
      if (cur >= 0) flush();
      cur = mid;
    }
    if (j0 + lane < wend) acc += prob64(a[i0 | (unsigned long long)lane]);
  }
  if (cur >= 0) flush();
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += kMarginalThreads) {
    double s = 0.0;
    for (int ww = 0; ww < kMarginalWarps; ++ww) s += hist[ww * nb + b];
    partial[(size_t)blockIdx.x * nb + b] = s;
  }
}

struct MarginalFinishArgs {
  int k, nl, C, pad;
  int dest[kMarginalMaxQubits];  // bit j of m -> (group << 8) | rank
};

__global__ void k_marginal_finish(const double *__restrict__ partial,
                                  const __grid_constant__ MarginalFinishArgs f,
                                  double *__restrict__ out) {
  const unsigned total = 1u << f.k;
  for (unsigned m = blockIdx.x * blockDim.x + threadIdx.x; m < total;
       m += gridDim.x * blockDim.x) {
    unsigned g = 0, b = 0;
    for (int j = 0; j < f.k; ++j) {
      const unsigned bit = (m >> j) & 1u;
      const int d = f.dest[j];
      if (d >> 8) g |= bit << (d & 255);
      else b |= bit << (d & 255);
    }
    const size_t nb = (size_t)1 << f.nl;
    double s = 0.0;
    for (int c = 0; c < f.C; ++c) s += partial[((size_t)g * f.C + c) * nb + b];
    out[m] = s;
  }
}

// Queue the marginal of `qubits` into device memory; *dout points into the
// state's staging buffer (valid until the next staging user).
static int marginal_device(qvmg_state s, int k, const int *qubits, double **dout) {
  if (k < 0 || k > kMarginalMaxQubits || k > s->nq)
    return fail(QVMG_E_INVALID, "marginal: 0 <= k <= min(20, qubits) required");
  if (k > 0 && !qubits) return fail(QVMG_E_INVALID, "null qubits");
  std::vector<int> sorted(qubits, qubits + k);
  for (int q : sorted)
    if (q < 0 || q >= s->nq) return fail(QVMG_E_INVALID, "marginal: qubit out of range");
  std::sort(sorted.begin(), sorted.end());
  for (int j = 1; j < k; ++j)
    if (sorted[j] == sorted[j - 1]) return fail(QVMG_E_INVALID, "marginal: repeated qubit");
  MarginalArgs p{};
  p.nl = std::min(k, kMarginalLocalMax);
  p.kh = k - p.nl;
  for (int r = 0; r < p.nl; ++r) p.lpos[r] = sorted[r];
  for (int r = 0; r < p.kh; ++r) p.gpos[r] = sorted[p.nl + r];
  const int groups = 1 << p.kh;
  p.count = s->len >> p.kh;
  unsigned long long C = std::max(1, kMarginalCtas / groups);
  C = std::min<unsigned long long>(C, std::max<unsigned long long>(1, p.count >> 8));
  p.C = (int)C;
  p.R = p.count / C;
  p.wlen = std::max<unsigned long long>(32, ((p.R / kMarginalWarps) + 31) & ~31ull);
  const size_t nb = (size_t)1 << p.nl;
  const size_t npartial = (size_t)groups * C * nb;
  const size_t nout = (size_t)1 << k;
  int rc = ensure_staging(s, (npartial + nout) * sizeof(double));
  if (rc) return rc;
  double *partial = (double *)s->staging;
  double *out = partial + npartial;
  const size_t smem = kMarginalWarps * nb * sizeof(double);
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  QVMG_CUDA(once(attr_once, attr_err, [] {
    const int bytes = kMarginalWarps * (1 << kMarginalLocalMax) * 8;
    cudaError_t e =
        cudaFuncSetAttribute(k_marginal<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_marginal<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               bytes);
    return e;
  }));
  const unsigned grid = (unsigned)(groups * C);
  if (s->prec == QVMG_FP64)
    k_marginal<double2><<<grid, kMarginalThreads, smem, s->stream>>>((const double2 *)s->amps, p,
                                                                     partial);
  else
    k_marginal<float2><<<grid, kMarginalThreads, smem, s->stream>>>((const float2 *)s->amps, p,
                                                                    partial);
  QVMG_CHECK_LAUNCH("k_marginal");
  MarginalFinishArgs f{};
  f.k = k;
  f.nl = p.nl;
  f.C = p.C;
  for (int j = 0; j < k; ++j) {
    const int r = (int)(std::lower_bound(sorted.begin(), sorted.end(), qubits[j]) - sorted.begin());
    f.dest[j] = r < p.nl ? r : (256 | (r - p.nl));
  }
  k_marginal_finish<<<(unsigned)std::min<size_t>((nout + 255) / 256, 1024), 256, 0, s->stream>>>(
      partial, f, out);
  QVMG_CHECK_LAUNCH("k_marginal_finish");
  *dout = out;
  return QVMG_OK;
}

// ---- big-endian wire bytes ---------------------------------------------------------

__device__ __forceinline__ unsigned long long bswap64(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned lo = (unsigned)u, hi = (unsigned)(u >> 32);
  return ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
}

template <typename C>
__global__ void k_wire_amps(const C *__restrict__ a, ulonglong2 *__restrict__ out, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const C v = a[i];
    out[i] = make_ulonglong2(bswap64((double)v.x), bswap64((double)v.y));
  }
}

template <typename C>
__global__ void k_wire_probs(const C *__restrict__ a, unsigned long long *__restrict__ out,
                             uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = bswap64(prob_f64(a[i]));  // the values qvmg_probabilities returns
}

static int produce_wire(qvmg_state s, uint64_t off, uint64_t n, void *dst, void *ctx) {
  const int probs = *static_cast<const int *>(ctx);
  const int grid = grid_for(n, 256);
  if (probs) {
    if (s->prec == QVMG_FP64)
      k_wire_probs<double2><<<grid, 256, 0, s->stream>>>((const double2 *)s->amps + off,
                                                          (unsigned long long *)dst, n);
    else
      k_wire_probs<float2><<<grid, 256, 0, s->stream>>>((const float2 *)s->amps + off,
                                                         (unsigned long long *)dst, n);
  } else {
    if (s->prec == QVMG_FP64)
      k_wire_amps<double2><<<grid, 256, 0, s->stream>>>((const double2 *)s->amps + off,
                                                         (ulonglong2 *)dst, n);
    else
      k_wire_amps<float2><<<grid, 256, 0, s->stream>>>((const float2 *)s->amps + off,
                                                        (ulonglong2 *)dst, n);
  }
  QVMG_CHECK_LAUNCH("k_wire");
  return QVMG_OK;
}

static int wire_stream(qvmg_state s, uint8_t *out, int probs) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!out) return fail(QVMG_E_INVALID, "null output");
  return stream_to_host(s, s->len, probs ? 8 : 16, out, produce_wire, &probs);
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

int qvmg_marginal_probabilities(qvmg_state s, int k, const int *qubits, double *out) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!out) return fail(QVMG_E_INVALID, "null output");
  double *dout = nullptr;
  if ((rc = marginal_device(s, k, qubits, &dout))) return rc;
  QVMG_CUDA(cudaMemcpyAsync(out, dout, ((size_t)1 << k) * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

int qvmg_measure_sequence(qvmg_state s, int k, const int *qubits, int convention, int ntrials,
                          const double *draws, uint64_t ndraws, uint8_t *bits,
                          uint64_t *draws_used) {
  int rc = check_state(s);
  if (rc) return rc;
  if (k < 0 || ntrials < 0) return fail(QVMG_E_INVALID, "negative count");
  if (convention != QVMG_MEASURE_INTERPRETED && convention != QVMG_MEASURE_COMPILED)
    return fail(QVMG_E_INVALID, "unknown measurement convention");
  if ((k > 0 && !qubits) || (k > 0 && ntrials > 0 && !bits))
    return fail(QVMG_E_INVALID, "null argument");
  if (ndraws > 0 && !draws) return fail(QVMG_E_INVALID, "null draws");
  // distinct measured qubits in order of first appearance
  std::vector<int> rank(s->nq, -1), order;
  for (int e = 0; e < k; ++e) {
    const int q = qubits[e];
    if (q == -1) continue;
    if (q < -1 || q >= s->nq) return fail(QVMG_E_INVALID, "measure sequence: qubit out of range");
    if (rank[q] < 0) {
      rank[q] = (int)order.size();
      order.push_back(q);
    }
  }
  const int kd = (int)order.size();
  if (kd > kMarginalMaxQubits)
    return fail(QVMG_E_UNSUPPORTED,
                "measure sequence: more than 20 distinct qubits (sample all qubits instead)");
  std::vector<double> table((size_t)1 << kd);
  if ((rc = qvmg_marginal_probabilities(s, kd, order.data(), table.data()))) return rc;
  // M[j][x]: probability that the first j measured qubits read x
  std::vector<std::vector<double>> M(kd + 1);
  M[kd] = std::move(table);
  for (int j = kd - 1; j >= 0; --j) {
    M[j].resize((size_t)1 << j);
    for (size_t x = 0; x < M[j].size(); ++x) M[j][x] = M[j + 1][x] + M[j + 1][x | ((size_t)1 << j)];
  }
  uint64_t used = 0;
  for (int t = 0; t < ntrials; ++t) {
    size_t prefix = 0;
    int nmeasured = 0;
    for (int e = 0; e < k; ++e) {
      const int q = qubits[e];
      int b = 0;
      if (q >= 0) {
        const int r = rank[q];
        double p1, p0;
        if (r < nmeasured) {  // measured before in this trial: deterministic
          p1 = (double)((prefix >> r) & 1u);
          p0 = 1.0 - p1;
        } else {
          const double denom = M[r][prefix];
          p1 = M[r + 1][prefix | ((size_t)1 << r)] / denom;
          p0 = M[r + 1][prefix] / denom;
        }
        if (convention == QVMG_MEASURE_INTERPRETED) {
          if (p1 != 0.0) {
            if (used >= ndraws) return fail(QVMG_E_RANGE, "measure sequence: out of draws");
            b = draws[used++] <= p1 ? 1 : 0;
          }
        } else {
          if (used >= ndraws) return fail(QVMG_E_RANGE, "measure sequence: out of draws");
          b = draws[used++] < p0 ? 0 : 1;
        }
        if (r == nmeasured) {
          prefix |= (size_t)b << r;
          ++nmeasured;
        }
      }
      bits[(size_t)t * k + e] = (uint8_t)b;
    }
  }
  if (draws_used) *draws_used = used;
  return QVMG_OK;
}

int qvmg_wavefunction_octets(qvmg_state s, uint8_t *out) { return wire_stream(s, out, 0); }

int qvmg_probabilities_octets(qvmg_state s, uint8_t *out) { return wire_stream(s, out, 1); }

}  // extern "C"
