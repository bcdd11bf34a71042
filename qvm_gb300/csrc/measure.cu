// measure.cu -- probability reductions, measurement, collapse and sampling.
//
// Replaces src/wavefunction.lisp:44-70 (ground/excited-state probability),
// :332-364 (norm, normalize), :382-395 (CDF), src/measurement.lisp:10-41
// (force-measurement), :87-105 (measure), :128-143 (measure-all-state),
// :179-225 (bisection sampler), :246-288 (CDF multishot sampler),
// src/compile-gate.lisp:221-254 (compiled measurement) and the inner
// product of app/src/api/expectation.lisp:80-84.
//
// All probability sums accumulate in FP64 over a fixed grid
// (kReduceBlocks x kReduceThreads) and a fixed combination tree, so a sum is
// bit-identical from run to run.  FP32 states form |a|^2 in FP32 and add it
// into a double-float (hi, lo) pair for short runs that are flushed to an
// FP64 accumulator, which keeps the FP64 pipe (1/64 of the FP32 rate on
// this part) out of the inner loop.
//
// Sampling is a two-level CDF: per-block FP64 sums over blocks of
// 2^kSampleBlockBits amplitudes, an inclusive FP64 prefix scan over the
// blocks, then one warp per draw binary-searches the block prefix and scans
// inside the block with warp shuffles.  The measurement decision (draw vs.
// probability) is taken on the device, so a measurement needs no host
// round trip between the reduction and the collapse.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

// ---- accumulation helpers ----------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum in a fixed order; result valid in thread 0.
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < THREADS / 32 ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Sum of |a_i|^2 over the amplitudes selected by `mode`:
// mode 0: all; mode 1: bit q == 0; mode 2: bit q == 1.
template <typename T>
__device__ __forceinline__ uint64_t sel_addr(uint64_t i, int mode, int q) {
  if (mode == 0) return i;
  uint64_t a = inject0(i, q);
  return mode == 2 ? (a | (1ull << q)) : a;
}

__global__ void __launch_bounds__(kReduceThreads)
    k_prob_sum_f64(const double2 *__restrict__ a, uint64_t count, int mode, int q,
                   double *__restrict__ partials) {
  __shared__ double sh[kReduceThreads / 32];
  double acc = 0.0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    acc += amp_prob(a[sel_addr<double>(i, mode, q)]);
  double r = block_sum<kReduceThreads>(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

__global__ void __launch_bounds__(kReduceThreads)
    k_prob_sum_f32(const float2 *__restrict__ a, uint64_t count, int mode, int q,
                   double *__restrict__ partials) {
  __shared__ double sh[kReduceThreads / 32];
  double acc = 0.0;
  float hi = 0.f, lo = 0.f;
  int run = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    df_add_prob(hi, lo, a[sel_addr<float>(i, mode, q)]);
    if (++run == 64) {
      acc += (double)hi + (double)lo;
      hi = lo = 0.f;
      run = 0;
    }
  }
  acc += (double)hi + (double)lo;
  double r = block_sum<kReduceThreads>(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

// Finish a reduction and take the measurement decision.
// what: 0 = plain sum (res->prob = sum)
//       1 = interpreted measure (sum is p1)
//       2 = compiled measure (sum is p0)
//       3 = norm (res->prob = sum, inv_norm = 1/sqrt(sum))
__global__ void k_finish(const double *__restrict__ partials, int nparts, int what,
                         double draw, MeasResult *__restrict__ res) {
  __shared__ double sh[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += partials[i];
  // blockDim.x == 1024
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double r = sh[lane];
    r = warp_sum(r);
    if (lane == 0) {
      res->prob = r;
      res->status = 0;
      if (what == 1) {
        // src/measurement.lisp:93-103
        double p1 = r;
        int bit, used;
        if (p1 == 0.0) {
          bit = 0;
          used = 0;
        } else {
          used = 1;
          bit = (draw <= p1) ? 1 : 0;
        }
        res->bit = bit;
        res->draw_used = used;
        res->inv_norm = bit ? 1.0 / sqrt(p1) : 1.0 / sqrt(1.0 - p1);
      } else if (what == 2) {
        // src/compile-gate.lisp:231-240
        double p0 = r;
        int keep_zero = draw < p0;
        res->bit = keep_zero ? 0 : 1;
        res->draw_used = 1;
        res->inv_norm = keep_zero ? 1.0 / sqrt(p0) : 1.0 / sqrt(1.0 - p0);
      } else if (what == 3) {
        res->inv_norm = 1.0 / sqrt(r);
      }
    }
  }
}

// force-measurement (src/measurement.lisp:26-39): one pass; amplitudes of
// the annihilated half are written as zero without being read.
template <typename T>
__global__ void __launch_bounds__(256)
    k_collapse(typename CT<T>::C *__restrict__ a, uint64_t len, int q,
               const MeasResult *__restrict__ res) {
  const int bit = res->bit;
  const T inv = (T)res->inv_norm;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if ((int)((i >> q) & 1ull) != bit) {
      a[i] = CT<T>::make(0, 0);
    } else {
      typename CT<T>::C v = a[i];
      v.x *= inv;
      v.y *= inv;
      a[i] = v;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_scale(typename CT<T>::C *__restrict__ a, uint64_t len, const MeasResult *__restrict__ res) {
  const T inv = (T)res->inv_norm;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len;
       i += (uint64_t)gridDim.x * blockDim.x) {
    typename CT<T>::C v = a[i];
    v.x *= inv;
    v.y *= inv;
    a[i] = v;
  }
}

// ---- two-level CDF -----------------------------------------------------------------
// Block sums: one CTA per sample block (grid-stride), fixed order.
template <typename T>
__global__ void __launch_bounds__(256)
    k_block_sums(const typename CT<T>::C *__restrict__ a, uint64_t nblocks, int block_bits,
                 double *__restrict__ sums) {
  __shared__ double sh[8];
  const uint64_t bsize = 1ull << block_bits;
  for (uint64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
    const typename CT<T>::C *p = a + b * bsize;
    double acc = 0.0;
    if constexpr (sizeof(T) == 4) {
      float hi = 0.f, lo = 0.f;
      for (uint64_t j = threadIdx.x; j < bsize; j += blockDim.x) df_add_prob(hi, lo, p[j]);
      acc = (double)hi + (double)lo;
    } else {
      for (uint64_t j = threadIdx.x; j < bsize; j += blockDim.x) acc += prob_f64(p[j]);
    }
    double r = block_sum<256>(acc, sh);
    if (threadIdx.x == 0) sums[b] = r;
  }
}

// Inclusive prefix scan in place over n doubles, one CTA of 1024 threads.
// The array is walked in coalesced tiles of 1024 consecutive entries: each
// tile is scanned by warp shuffles and a scan of the 32 warp totals, shifted
// by the running total of the tiles before it; the next tile's load is issued
// before the current one is scanned.  (The block-sum array is at most 2^18+1
// entries for a 30-qubit state, 2 MiB, and stays in L2.)
__global__ void __launch_bounds__(1024) k_scan_inclusive(double *__restrict__ x, uint64_t n) {
  __shared__ double warp_tot[32];
  __shared__ double carry_sh;
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double carry = 0.0;
  double next = threadIdx.x < n ? x[threadIdx.x] : 0.0;
  for (uint64_t base = 0; base < n; base += 1024) {
    const uint64_t i = base + threadIdx.x;
    double v = next;
    next = base + 1024 + threadIdx.x < n ? x[base + 1024 + threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= (unsigned)o) v += y;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
      double t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= (unsigned)o) t += y;
      }
      warp_tot[lane] = t;  // inclusive scan of the warp totals
      if (lane == 31) carry_sh = t;
    }
    __syncthreads();
    const double before = warp ? warp_tot[warp - 1] : 0.0;
    if (i < n) x[i] = carry + (before + v);
    carry += carry_sh;
    __syncthreads();  // warp_tot and carry_sh are rewritten by the next tile
  }
}

// One warp per draw.  rule 0 (bisection): smallest b in [0, len-2] with
// C(b) > p, else len-1.  rule 1 (CDF): smallest i with C(i) >= p, else len-1.
template <typename T>
__global__ void __launch_bounds__(256)
    k_sample(const typename CT<T>::C *__restrict__ a, uint64_t len, int block_bits,
             const double *__restrict__ prefix, uint64_t nblocks,
             const double *__restrict__ draws, uint64_t nshots, int rule,
             unsigned long long *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t t = warp; t < nshots; t += nwarps) {
    // FP32 states sample the renormalised distribution: their norm drifts by
    // ~1e-7 over a deep circuit, which would shift the whole CDF; FP64 states
    // use the draw as is, like the reference.
    const double p = sizeof(T) == 4 ? draws[t] * prefix[nblocks - 1] : draws[t];
    // First block whose inclusive prefix passes p.
    uint64_t lo = 0, hi = nblocks;  // search in [lo, hi)
    while (lo < hi) {
      uint64_t mid = lo + (hi - lo) / 2;
      double c = prefix[mid];
      bool pass = rule == 0 ? (c > p) : (c >= p);
      if (pass) hi = mid; else lo = mid + 1;
    }
    unsigned long long result = len - 1;
    if (lo < nblocks) {
      const uint64_t b = lo;
      const uint64_t bsize = 1ull << block_bits;
      double run = b ? prefix[b - 1] : 0.0;
      const typename CT<T>::C *blk = a + b * bsize;
      result = b * bsize + bsize - 1;  // rounding fallback: block's last index
      for (uint64_t c0 = 0; c0 < bsize; c0 += 32) {
        // blocks of states below 5 qubits are shorter than a warp
        const bool valid = c0 + lane < bsize;
        double pr = valid ? prob_f64(blk[c0 + lane]) : 0.0;
        // inclusive warp scan
        double sc = pr;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          double y = __shfl_up_sync(0xffffffffu, sc, o);
          if (lane >= o) sc += y;
        }
        double c = run + sc;
        bool pass = valid && (rule == 0 ? (c > p) : (c >= p));
        unsigned m = __ballot_sync(0xffffffffu, pass);
        if (m) {
          result = b * bsize + c0 + (__ffs(m) - 1);
          break;
        }
        run += __shfl_sync(0xffffffffu, sc, 31);
      }
      if (rule == 0 && result > len - 1) result = len - 1;
    }
    if (rule == 0 && result == len - 1) {
      // the bisection never evaluates C(len-1); nothing to adjust.
    }
    if (lane == 0) out[t] = result;
  }
}

template <typename T>
__global__ void k_set_basis(typename CT<T>::C *__restrict__ a, const unsigned long long *idx) {
  a[*idx] = CT<T>::make(1, 0);
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_probs(const typename CT<T>::C *__restrict__ a, double *__restrict__ out, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    out[i] = prob_f64(a[i]);
  }
}

// sum conj(a_i) b_i, max |a_i - b_i|, |a|^2 and |b|^2 over two states of
// equal length: 5 partials per block.
template <typename TA, typename TB>
__global__ void __launch_bounds__(kReduceThreads)
    k_inner(const typename CT<TA>::C *__restrict__ a, const typename CT<TB>::C *__restrict__ b,
            uint64_t len, double *__restrict__ partials) {
  __shared__ double sh[kReduceThreads / 32];
  double re = 0.0, im = 0.0, mx = 0.0, na = 0.0, nb = 0.0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len;
       i += (uint64_t)gridDim.x * blockDim.x) {
    typename CT<TA>::C x = a[i];
    typename CT<TB>::C y = b[i];
    double xr = x.x, xi = x.y, yr = y.x, yi = y.y;
    re += xr * yr + xi * yi;
    im += xr * yi - xi * yr;
    na += xr * xr + xi * xi;
    nb += yr * yr + yi * yi;
    double dr = xr - yr, di = xi - yi;
    mx = fmax(mx, sqrt(dr * dr + di * di));
  }
  double r = block_sum<kReduceThreads>(re, sh);
  double s = block_sum<kReduceThreads>(im, sh);
  double sa = block_sum<kReduceThreads>(na, sh);
  double sb = block_sum<kReduceThreads>(nb, sh);
  // block max
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = mx;
  __syncthreads();
  if (w == 0) {
    double m = lane < kReduceThreads / 32 ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) {
      double *q = partials + 5 * blockIdx.x;
      q[0] = r;
      q[1] = s;
      q[2] = m;
      q[3] = sa;
      q[4] = sb;
    }
  }
}

__global__ void k_finish_inner(const double *__restrict__ partials, int nparts,
                               MeasResult *__restrict__ res) {
  // single thread, fixed order (nparts is small)
  double re = 0.0, im = 0.0, mx = 0.0, na = 0.0, nb = 0.0;
  for (int i = 0; i < nparts; ++i) {
    const double *q = partials + 5 * i;
    re += q[0];
    im += q[1];
    mx = fmax(mx, q[2]);
    na += q[3];
    nb += q[4];
  }
  res->prob = re;
  res->aux = im;
  res->inv_norm = mx;
  res->na = na;
  res->nb = nb;
}

// ---- host helpers ---------------------------------------------------------------------

// Reduce |a|^2 over the selected half (mode 1/2) or everything (mode 0);
// then finish with decision `what` using `draw`.  Leaves the result in dres.
static int reduce_and_finish(qvmg_state s, int mode, int q, int what, double draw) {
  uint64_t count = mode == 0 ? s->len : s->len / 2;
  if (s->prec == QVMG_FP64)
    k_prob_sum_f64<<<kReduceBlocks, kReduceThreads, 0, s->stream>>>(
        (const double2 *)s->amps, count, mode, q, s->partials);
  else
    k_prob_sum_f32<<<kReduceBlocks, kReduceThreads, 0, s->stream>>>(
        (const float2 *)s->amps, count, mode, q, s->partials);
  QVMG_CHECK_LAUNCH("k_prob_sum");
  k_finish<<<1, 1024, 0, s->stream>>>(s->partials, kReduceBlocks, what, draw, s->dres);
  QVMG_CHECK_LAUNCH("k_finish");
  return QVMG_OK;
}

static int fetch_result(qvmg_state s) {
  QVMG_CUDA(cudaMemcpyAsync(s->hres, s->dres, sizeof(MeasResult), cudaMemcpyDeviceToHost,
                            s->stream));
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

static int collapse(qvmg_state s, int q) {
  int grid = grid_for(s->len, 256);
  if (s->prec == QVMG_FP64)
    k_collapse<double><<<grid, 256, 0, s->stream>>>((double2 *)s->amps, s->len, q, s->dres);
  else
    k_collapse<float><<<grid, 256, 0, s->stream>>>((float2 *)s->amps, s->len, q, s->dres);
  QVMG_CHECK_LAUNCH("k_collapse");
  return QVMG_OK;
}

static int check_qubit(qvmg_state s, int q) {
  if (q < 0 || q >= s->nq)
    return fail(QVMG_E_INVALID, "Trying to measure qubit " + std::to_string(q) + " on a QVM with only " +
                                    std::to_string(s->nq) + " qubits.");
  return QVMG_OK;
}

// Build block prefix sums (inclusive) into s->block_sums.
static int build_cdf(qvmg_state s, int *block_bits_out) {
  int bb = s->nq > kSampleBlockBits ? kSampleBlockBits : s->nq;
  uint64_t nblocks = s->len >> bb;
  int grid = (int)std::min<uint64_t>(nblocks, (uint64_t)sm_count() * 8);
  if (s->prec == QVMG_FP64)
    k_block_sums<double><<<grid, 256, 0, s->stream>>>((const double2 *)s->amps, nblocks, bb,
                                                      s->block_sums);
  else
    k_block_sums<float><<<grid, 256, 0, s->stream>>>((const float2 *)s->amps, nblocks, bb,
                                                     s->block_sums);
  QVMG_CHECK_LAUNCH("k_block_sums");
  k_scan_inclusive<<<1, 1024, 0, s->stream>>>(s->block_sums, nblocks);
  QVMG_CHECK_LAUNCH("k_scan_inclusive");
  *block_bits_out = bb;
  return QVMG_OK;
}

static int sample_device(qvmg_state s, const double *d_draws, uint64_t nshots, int rule,
                         unsigned long long *d_out) {
  int bb = 0;
  int rc = build_cdf(s, &bb);
  if (rc) return rc;
  uint64_t nblocks = s->len >> bb;
  int grid = grid_for(nshots * 32, 256);
  if (s->prec == QVMG_FP64)
    k_sample<double><<<grid, 256, 0, s->stream>>>((const double2 *)s->amps, s->len, bb,
                                                  s->block_sums, nblocks, d_draws, nshots,
                                                  rule, d_out);
  else
    k_sample<float><<<grid, 256, 0, s->stream>>>((const float2 *)s->amps, s->len, bb,
                                                 s->block_sums, nblocks, d_draws, nshots,
                                                 rule, d_out);
  QVMG_CHECK_LAUNCH("k_sample");
  return QVMG_OK;
}

// The inner-product partials need 3 doubles per block; the partial buffer
// holds 2*kReduceBlocks doubles, so the inner kernel uses a third of the
// blocks' worth of space via dvec instead.
static int inner_impl(qvmg_state a, qvmg_state b) {
  int rc = order_states(a, b);
  if (rc) return rc;
  if ((rc = ensure_dvec(a, 5 * kReduceBlocks * sizeof(double)))) return rc;
  double *parts = a->dvec;
  auto go = [&](auto ta, auto tb) {
    using TA = decltype(ta);
    using TB = decltype(tb);
    k_inner<TA, TB><<<kReduceBlocks, kReduceThreads, 0, a->stream>>>(
        (const typename CT<TA>::C *)a->amps, (const typename CT<TB>::C *)b->amps, a->len,
        parts);
  };
  if (a->prec == QVMG_FP64 && b->prec == QVMG_FP64) go(0.0, 0.0);
  else if (a->prec == QVMG_FP64) go(0.0, 0.0f);
  else if (b->prec == QVMG_FP64) go(0.0f, 0.0);
  else go(0.0f, 0.0f);
  QVMG_CHECK_LAUNCH("k_inner");
  k_finish_inner<<<1, 1, 0, a->stream>>>(parts, kReduceBlocks, a->dres);
  QVMG_CHECK_LAUNCH("k_finish_inner");
  if ((rc = fetch_result(a))) return rc;
  return order_states(b, a);
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

int qvmg_prob_excited(qvmg_state s, int q, double *p1) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubit(s, q))) return rc;
  if ((rc = reduce_and_finish(s, 2, q, 0, 0.0))) return rc;
  if ((rc = fetch_result(s))) return rc;
  if (p1) *p1 = s->hres->prob;
  return QVMG_OK;
}

int qvmg_prob_ground(qvmg_state s, int q, double *p0) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubit(s, q))) return rc;
  if ((rc = reduce_and_finish(s, 1, q, 0, 0.0))) return rc;
  if ((rc = fetch_result(s))) return rc;
  if (p0) *p0 = s->hres->prob;
  return QVMG_OK;
}

int qvmg_force_measurement(qvmg_state s, int q, int bit, double p1) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubit(s, q))) return rc;
  if (bit != 0 && bit != 1) return fail(QVMG_E_INVALID, "measured value must be 0 or 1");
  double keep = bit ? p1 : 1.0 - p1;
  if (!(keep > 0.0) || !(p1 >= 0.0) || !(p1 <= 1.0))
    return fail(QVMG_E_RANGE, "cannot force qubit " + std::to_string(q) + " to " +
                                  std::to_string(bit) + " with excited probability " +
                                  std::to_string(p1));
  // hres is the pinned source of a queued copy: let earlier copies finish.
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  MeasResult r{};
  r.bit = bit;
  r.prob = p1;
  r.inv_norm = 1.0 / sqrt(keep);
  *s->hres = r;
  QVMG_CUDA(cudaMemcpyAsync(s->dres, s->hres, sizeof(MeasResult), cudaMemcpyHostToDevice,
                            s->stream));
  return collapse(s, q);
}

int qvmg_measure(qvmg_state s, int q, double draw, int convention, int *bit, int *draw_used,
                 double *prob) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubit(s, q))) return rc;
  if (convention != QVMG_MEASURE_INTERPRETED && convention != QVMG_MEASURE_COMPILED)
    return fail(QVMG_E_INVALID, "unknown measurement convention");
  if (convention == QVMG_MEASURE_INTERPRETED)
    rc = reduce_and_finish(s, 2, q, 1, draw);
  else
    rc = reduce_and_finish(s, 1, q, 2, draw);
  if (rc) return rc;
  if ((rc = collapse(s, q))) return rc;
  if ((rc = fetch_result(s))) return rc;
  if (bit) *bit = s->hres->bit;
  if (draw_used) *draw_used = s->hres->draw_used;
  if (prob) *prob = s->hres->prob;
  return QVMG_OK;
}

int qvmg_measure_all(qvmg_state s, double draw, uint64_t *index) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = ensure_dvec(s, 64))) return rc;
  // draw at dvec[0], result index at dres->index
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  s->hres->prob = draw;
  QVMG_CUDA(cudaMemcpyAsync(s->dvec, &s->hres->prob, sizeof(double), cudaMemcpyHostToDevice,
                            s->stream));
  unsigned long long *d_idx = &s->dres->index;
  if ((rc = sample_device(s, s->dvec, 1, 0, d_idx))) return rc;
  QVMG_CUDA(cudaMemsetAsync(s->amps, 0, s->len * amp_bytes(s->prec), s->stream));
  if (s->prec == QVMG_FP64)
    k_set_basis<double><<<1, 1, 0, s->stream>>>((double2 *)s->amps, d_idx);
  else
    k_set_basis<float><<<1, 1, 0, s->stream>>>((float2 *)s->amps, d_idx);
  QVMG_CHECK_LAUNCH("k_set_basis");
  if ((rc = fetch_result(s))) return rc;
  if (index) *index = s->hres->index;
  return QVMG_OK;
}

int qvmg_sample(qvmg_state s, const double *draws, uint64_t nshots, int rule, uint64_t *out) {
  int rc = check_state(s);
  if (rc) return rc;
  if (rule != QVMG_SAMPLE_BISECT && rule != QVMG_SAMPLE_CDF)
    return fail(QVMG_E_INVALID, "unknown sampling rule");
  if (nshots == 0) return QVMG_OK;
  if (!draws || !out) return fail(QVMG_E_INVALID, "null draws or output");
  for (uint64_t i = 0; i < nshots; ++i)
    if (!(draws[i] >= 0.0 && draws[i] <= 1.0))
      return fail(QVMG_E_INVALID, "draw outside [0, 1]");
  uint64_t bytes = nshots * 16;
  if ((rc = ensure_dvec(s, bytes))) return rc;
  double *d_draws = s->dvec;
  unsigned long long *d_out = (unsigned long long *)(s->dvec + nshots);
  QVMG_CUDA(cudaMemcpyAsync(d_draws, draws, nshots * 8, cudaMemcpyHostToDevice, s->stream));
  if ((rc = sample_device(s, d_draws, nshots, rule, d_out))) return rc;
  QVMG_CUDA(cudaMemcpyAsync(out, d_out, nshots * 8, cudaMemcpyDeviceToHost, s->stream));
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

static int produce_probs(qvmg_state s, uint64_t off, uint64_t n, void *dst, void *) {
  if (s->prec == QVMG_FP64)
    k_probs<double><<<grid_for(n, 256), 256, 0, s->stream>>>((const double2 *)s->amps + off,
                                                             (double *)dst, n);
  else
    k_probs<float><<<grid_for(n, 256), 256, 0, s->stream>>>((const float2 *)s->amps + off,
                                                            (double *)dst, n);
  QVMG_CHECK_LAUNCH("k_probs");
  return QVMG_OK;
}

int qvmg_probabilities(qvmg_state s, double *out) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!out) return fail(QVMG_E_INVALID, "null output");
  return stream_to_host(s, s->len, 8, out, produce_probs, nullptr);
}

int qvmg_norm(qvmg_state s, double *norm) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = reduce_and_finish(s, 0, 0, 3, 0.0))) return rc;
  if ((rc = fetch_result(s))) return rc;
  if (norm) *norm = sqrt(s->hres->prob);
  return QVMG_OK;
}

int qvmg_normalize(qvmg_state s) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = reduce_and_finish(s, 0, 0, 3, 0.0))) return rc;
  int grid = grid_for(s->len, 256);
  if (s->prec == QVMG_FP64)
    k_scale<double><<<grid, 256, 0, s->stream>>>((double2 *)s->amps, s->len, s->dres);
  else
    k_scale<float><<<grid, 256, 0, s->stream>>>((float2 *)s->amps, s->len, s->dres);
  QVMG_CHECK_LAUNCH("k_scale");
  return QVMG_OK;
}

int qvmg_inner(qvmg_state a, qvmg_state b, double *re, double *im) {
  int rc = check_state(a);
  if (rc) return rc;
  if ((rc = check_state(b))) return rc;
  if (a->nq != b->nq) return fail(QVMG_E_INVALID, "inner product of states of different sizes");
  if ((rc = inner_impl(a, b))) return rc;
  if (re) *re = a->hres->prob;
  if (im) *im = a->hres->aux;
  return QVMG_OK;
}

int qvmg_fidelity(qvmg_state a, qvmg_state b, double *fidelity, double *max_abs_err) {
  int rc = check_state(a);
  if (rc) return rc;
  if ((rc = check_state(b))) return rc;
  if (a->nq != b->nq) return fail(QVMG_E_INVALID, "fidelity of states of different sizes");
  if ((rc = inner_impl(a, b))) return rc;
  double re = a->hres->prob, im = a->hres->aux;
  // fidelity of the normalised states: |<a|b>|^2 / (<a|a><b|b>)
  if (fidelity) *fidelity = (re * re + im * im) / (a->hres->na * a->hres->nb);
  if (max_abs_err) *max_abs_err = a->hres->inv_norm;
  return QVMG_OK;
}

}  // extern "C"

// ---- sampling without any allocation ----------------------------------------------
//
// qvmg_sample needs a state handle, and creating one allocates device memory
// (the amplitudes and the per-state CDF scratch).  Some callers cannot do
// that: a host that hands the library a slice of its own pre-reserved device
// pool and forbids cudaMalloc (which synchronises the device and can fail
// under memory pressure in a long-running server), or a caller in the middle
// of a latency-critical loop where an allocation's implicit synchronisation
// is not acceptable.  qvmg_sample_noalloc serves them: the caller passes the
// amplitudes, the draws and the output as device pointers plus a stream, and
// the block sums of the two-level CDF live in the fixed array below, which
// every GPU that loads this library holds until the process exits.
namespace qvmg {

// Largest state the fixed scratch covers: 2^30 amplitudes.
constexpr int kNoAllocMaxQubits = 30;
constexpr uint64_t kNoAllocBlocks = 1ull << (kNoAllocMaxQubits - kSampleBlockBits);

// Block sums of the CDF (then their inclusive prefix), shared by all calls.
static __device__ __align__(256) double g_noalloc_cdf[kNoAllocBlocks + 1];

// Device address of g_noalloc_cdf per device ordinal, looked up once.
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[256];

static int noalloc_scratch(double **out) {
  int dev = 0;
  QVMG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail(QVMG_E_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_cdf);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_cdf)");
    g_noalloc_ptr[dev] = (double *)p;
  }
  *out = g_noalloc_ptr[dev];
  return QVMG_OK;
}

template <typename T>
static int sample_noalloc_impl(const void *amps, int n, const double *draws, uint64_t nshots,
                               int rule, unsigned long long *out, double *cdf,
                               cudaStream_t st) {
  using C = typename CT<T>::C;
  const uint64_t len = 1ull << n;
  const int bb = n > kSampleBlockBits ? kSampleBlockBits : n;
  const uint64_t nblocks = len >> bb;
  // Every entry of cdf[0..nblocks) is written by k_block_sums before the scan
  // reads it, so nothing left over from an earlier call is ever used.
  int grid = (int)std::min<uint64_t>(nblocks, (uint64_t)sm_count() * 8);
  k_block_sums<T><<<grid, 256, 0, st>>>((const C *)amps, nblocks, bb, cdf);
  QVMG_CHECK_LAUNCH("k_block_sums");
  k_scan_inclusive<<<1, 1024, 0, st>>>(cdf, nblocks);
  QVMG_CHECK_LAUNCH("k_scan_inclusive");
  k_sample<T><<<grid_for(nshots * 32, 256), 256, 0, st>>>((const C *)amps, len, bb, cdf, nblocks,
                                                          draws, nshots, rule, out);
  QVMG_CHECK_LAUNCH("k_sample");
  return QVMG_OK;
}

}  // namespace qvmg

extern "C" int qvmg_sample_noalloc(const void *amps, int nqubits, int precision,
                                   const double *draws, uint64_t nshots, int rule,
                                   uint64_t *out, void *stream) {
  if (nqubits < 1 || nqubits > kNoAllocMaxQubits)
    return fail(QVMG_E_INVALID, "qvmg_sample_noalloc: " + std::to_string(nqubits) +
                                    " qubits is outside 1.." +
                                    std::to_string(kNoAllocMaxQubits) +
                                    ", the size its fixed scratch covers");
  if (precision != QVMG_FP64 && precision != QVMG_FP32)
    return fail(QVMG_E_INVALID, "qvmg_sample_noalloc: precision must be QVMG_FP64 or QVMG_FP32");
  if (rule != QVMG_SAMPLE_BISECT && rule != QVMG_SAMPLE_CDF)
    return fail(QVMG_E_INVALID, "qvmg_sample_noalloc: unknown sampling rule");
  if (nshots == 0) return QVMG_OK;
  if (!amps || !draws || !out)
    return fail(QVMG_E_INVALID, "qvmg_sample_noalloc: null device pointer");
  double *cdf = nullptr;
  int rc = noalloc_scratch(&cdf);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == QVMG_FP64)
    return sample_noalloc_impl<double>(amps, nqubits, draws, nshots, rule,
                                       (unsigned long long *)out, cdf, st);
  return sample_noalloc_impl<float>(amps, nqubits, draws, nshots, rule,
                                    (unsigned long long *)out, cdf, st);
}
