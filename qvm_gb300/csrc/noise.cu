// noise.cu -- stochastic Kraus maps on a pure state; density-matrix diagonals.
//
// The reference's noisy QVM applies a noisy gate, given as a Kraus map
// {K_j}, to a pure state by inverse transform sampling
// (%evolve-pure-state-stochastically, src/apply-gate.lisp:16-39): draw r,
// then for j = 0, 1, ... copy the state, apply K_j to the copy, add
// p_j = ||K_j psi||^2 to a running sum, and stop at the first j whose sum
// reaches r; that copy, normalised, becomes the state.  That is up to one
// copy, one gate pass and one reduction per Kraus operator, then a
// normalisation.
//
// Here every p_j comes from one read of the state: p_j = tr(K_j rho K_j^H)
// with rho the reduced density matrix of the gate's qubits
// (rho[r][c] = sum over the other qubits of a_r conj(a_c)), reduced on the
// device in a fixed order.  The chosen K_j / sqrt(p_j) is then applied in
// one gate pass (which also normalises).  Two passes in all, independent of
// the number of Kraus operators.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

constexpr int kRdmMaxQubits = 2;

struct RdmArgs {
  int k;
  int sp[kRdmMaxQubits];      // sorted positions
  unsigned long long off[1 << kRdmMaxQubits];  // sub-index r -> address offset
  unsigned long long ngroups;
};

__device__ __forceinline__ double2 ld64(const double2 *a, unsigned long long i) { return a[i]; }
__device__ __forceinline__ double2 ld64(const float2 *a, unsigned long long i) {
  const float2 v = a[i];
  return make_double2(v.x, v.y);
}

// Per-block sums of the 4^K accumulators: rho diagonal, then (re, im) of
// rho[r][c] for r < c.
template <typename C, int K>
__global__ void __launch_bounds__(kReduceThreads)
    k_rdm(const C *__restrict__ a, const __grid_constant__ RdmArgs p, double *__restrict__ part) {
  constexpr int D = 1 << K, NA = D * D;
  __shared__ double sh[kReduceThreads / 32][NA];
  double acc[NA];
#pragma unroll
  for (int i = 0; i < NA; ++i) acc[i] = 0.0;
  for (unsigned long long g = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
       g < p.ngroups; g += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long base = g;
#pragma unroll
    for (int s = 0; s < K; ++s) base = inject0(base, p.sp[s]);
    double2 v[D];
#pragma unroll
    for (int r = 0; r < D; ++r) v[r] = ld64(a, base + p.off[r]);
#pragma unroll
    for (int r = 0; r < D; ++r) acc[r] = fma(v[r].x, v[r].x, fma(v[r].y, v[r].y, acc[r]));
    int i = D;
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int c = r + 1; c < D; ++c) {
        // v_r conj(v_c)
        acc[i] = fma(v[r].x, v[c].x, fma(v[r].y, v[c].y, acc[i]));
        acc[i + 1] = fma(v[r].y, v[c].x, fma(-v[r].x, v[c].y, acc[i + 1]));
        i += 2;
      }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NA; ++i) {
    double x = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[w][i] = x;
  }
  __syncthreads();
  if (threadIdx.x < NA) {
    double s = 0.0;
    for (int ww = 0; ww < kReduceThreads / 32; ++ww) s += sh[ww][threadIdx.x];
    part[(size_t)blockIdx.x * NA + threadIdx.x] = s;
  }
}

// rho (2^k x 2^k complex, row-major, interleaved re/im) of `qubits` (nat
// order: bit j of a row index <-> qubits[j]).
static int reduced_density_matrix(qvmg_state s, int k, const int *qubits, std::vector<double> &rho) {
  int rc = check_qubits(s, k, qubits, kRdmMaxQubits);
  if (rc) return rc;
  RdmArgs p{};
  p.k = k;
  std::vector<int> sp(qubits, qubits + k);
  std::sort(sp.begin(), sp.end());
  for (int j = 0; j < k; ++j) p.sp[j] = sp[j];
  const int D = 1 << k, NA = D * D;
  for (int r = 0; r < D; ++r) {
    unsigned long long o = 0;
    for (int j = 0; j < k; ++j)
      if ((r >> j) & 1) o |= 1ull << qubits[j];
    p.off[r] = o;
  }
  p.ngroups = s->len >> k;
  if ((rc = ensure_staging(s, (size_t)kReduceBlocks * NA * sizeof(double)))) return rc;
  double *part = (double *)s->staging;
  if (s->prec == QVMG_FP64) {
    if (k == 1) k_rdm<double2, 1><<<kReduceBlocks, kReduceThreads, 0, s->stream>>>((const double2 *)s->amps, p, part);
    else k_rdm<double2, 2><<<kReduceBlocks, kReduceThreads, 0, s->stream>>>((const double2 *)s->amps, p, part);
  } else {
    if (k == 1) k_rdm<float2, 1><<<kReduceBlocks, kReduceThreads, 0, s->stream>>>((const float2 *)s->amps, p, part);
    else k_rdm<float2, 2><<<kReduceBlocks, kReduceThreads, 0, s->stream>>>((const float2 *)s->amps, p, part);
  }
  QVMG_CHECK_LAUNCH("k_rdm");
  std::vector<double> host((size_t)kReduceBlocks * NA);
  QVMG_CUDA(cudaMemcpyAsync(host.data(), part, host.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, s->stream));
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  std::vector<double> sum(NA, 0.0);
  for (int b = 0; b < kReduceBlocks; ++b)
    for (int i = 0; i < NA; ++i) sum[i] += host[(size_t)b * NA + i];
  rho.assign((size_t)2 * NA, 0.0);
  for (int r = 0; r < D; ++r) rho[2 * (r * D + r)] = sum[r];
  int i = D;
  for (int r = 0; r < D; ++r)
    for (int c = r + 1; c < D; ++c) {
      rho[2 * (r * D + c)] = sum[i];
      rho[2 * (r * D + c) + 1] = sum[i + 1];
      rho[2 * (c * D + r)] = sum[i];
      rho[2 * (c * D + r) + 1] = -sum[i + 1];
      i += 2;
    }
  return QVMG_OK;
}

// ||K psi||^2 = tr(K rho K^H) = sum_r sum_{c,c'} K[r][c] rho[c][c'] conj(K[r][c']).
static double kraus_probability(const double *K, const std::vector<double> &rho, int D) {
  double total = 0.0;
  for (int r = 0; r < D; ++r) {
    double re = 0.0;
    for (int c = 0; c < D; ++c) {
      // t = sum_{c'} rho[c][c'] conj(K[r][c'])
      double tr = 0.0, ti = 0.0;
      for (int c2 = 0; c2 < D; ++c2) {
        const double pr = rho[2 * (c * D + c2)], pi = rho[2 * (c * D + c2) + 1];
        const double kr = K[2 * (r * D + c2)], ki = -K[2 * (r * D + c2) + 1];
        tr += pr * kr - pi * ki;
        ti += pr * ki + pi * kr;
      }
      const double ar = K[2 * (r * D + c)], ai = K[2 * (r * D + c) + 1];
      re += ar * tr - ai * ti;
    }
    total += re;
  }
  return total;
}

// ---- density matrices stored as 2n-qubit vectors ------------------------------------
//
// vec(rho) is row-major (src/state-representation.lisp:173-188,235-266):
// entry (i, j) of the 2^n x 2^n matrix is amplitude i * 2^n + j, so the
// diagonal is the stride-(2^n + 1) slice.
template <typename C>
__global__ void k_density_diagonal(const C *__restrict__ a, uint64_t dim, double *__restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (double)a[i * (dim + 1)].x;
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

int qvmg_reduced_density_matrix(qvmg_state s, int k, const int *qubits, double *rho) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!rho) return fail(QVMG_E_INVALID, "null output");
  if (k < 1 || k > kRdmMaxQubits) return fail(QVMG_E_UNSUPPORTED, "reduced density matrix: 1 <= k <= 2");
  std::vector<double> r;
  if ((rc = reduced_density_matrix(s, k, qubits, r))) return rc;
  std::copy(r.begin(), r.end(), rho);
  return QVMG_OK;
}

int qvmg_density_diagonal(qvmg_state s, double *out) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!out) return fail(QVMG_E_INVALID, "null output");
  if (s->nq % 2) return fail(QVMG_E_INVALID, "a density matrix needs an even qubit count");
  const uint64_t dim = 1ull << (s->nq / 2);
  if ((rc = ensure_staging(s, dim * sizeof(double)))) return rc;
  if (s->prec == QVMG_FP64)
    k_density_diagonal<double2><<<grid_for(dim, 256), 256, 0, s->stream>>>(
        (const double2 *)s->amps, dim, (double *)s->staging);
  else
    k_density_diagonal<float2><<<grid_for(dim, 256), 256, 0, s->stream>>>(
        (const float2 *)s->amps, dim, (double *)s->staging);
  QVMG_CHECK_LAUNCH("k_density_diagonal");
  QVMG_CUDA(cudaMemcpyAsync(out, s->staging, dim * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return QVMG_OK;
}

int qvmg_apply_kraus(qvmg_state s, int k, const int *qubits, int nops, const double *ops,
                     double draw, int *chosen, double *probability) {
  int rc = check_state(s);
  if (rc) return rc;
  if (k < 1 || k > kRdmMaxQubits) return fail(QVMG_E_UNSUPPORTED, "Kraus maps on 1 or 2 qubits");
  if (nops < 1 || !ops) return fail(QVMG_E_INVALID, "empty Kraus map");
  if (!(draw >= 0.0 && draw <= 1.0)) return fail(QVMG_E_INVALID, "draw outside [0, 1]");
  std::vector<double> rho;
  if ((rc = reduced_density_matrix(s, k, qubits, rho))) return rc;
  const int D = 1 << k;
  const size_t msz = (size_t)2 * D * D;
  // first j whose running sum reaches the draw; the last operator when
  // rounding leaves the total short of it (the loop then ends there)
  double summed = 0.0, pj = 0.0;
  int j = 0;
  for (; j < nops; ++j) {
    pj = kraus_probability(ops + j * msz, rho, D);
    summed += pj;
    if (summed >= draw) break;
  }
  if (j == nops) j = nops - 1;
  if (!(pj > 0.0))
    return fail(QVMG_E_RANGE, "the selected Kraus operator annihilates the state");
  const double scale = 1.0 / sqrt(pj);
  std::vector<double> m(ops + j * msz, ops + (j + 1) * msz);
  for (double &x : m) x *= scale;
  if ((rc = launch_dense(s, k, qubits, m.data()))) return rc;
  if (chosen) *chosen = j;
  if (probability) *probability = pj;
  return QVMG_OK;
}

}  // extern "C"
