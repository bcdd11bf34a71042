// gates.cu -- per-gate ("plain") kernels: one HBM pass per source gate.
//
// These replace the reference's apply-matrix-operator and its serial /
// AVX2 kernels (src/wavefunction.lisp:271-330, src/serial-kernels.lisp:
// 19-288, src/impl/sbcl-avx-vops.lisp) and the compiled permutation gates
// (src/compile-gate.lisp:259-309):
//  - k_dense<K>: for each of the 2^(n-K) groups (complement indices with K
//    zero bits injected, src/wavefunction.lisp:155-175), gather the 2^K
//    amplitudes into registers, multiply by the matrix held in the kernel's
//    parameter bank (uniform across the warp), scatter back.  128-bit loads
//    (one double2 / float2 per amplitude), grid-stride over groups.
//  - k_perm<K>: only the amplitudes a permutation moves are read/written.
//  - k_diag_tables_f32 / _f64: a run of diagonal gates is folded on the host
//    into at most kMaxTables phase tables over <= 10 qubits each (ascending
//    qubits; a contiguous range is indexed by one shift and mask); each
//    amplitude's phase is the product of its table entries other than 1;
//    amplitudes whose entries are all 1 are neither read nor written.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

template <typename T, int K>
struct DenseArgs {
  typename CT<T>::C m[(1 << K) * (1 << K)];  // row-major
  uint64_t off[1 << K];                      // address offset of sub-index c
  int sorted[K];                             // gate qubits, ascending
};

template <typename T, int K, bool REAL>
__global__ void __launch_bounds__(256)
    k_dense(typename CT<T>::C *__restrict__ a, uint64_t ngroups,
            const __grid_constant__ DenseArgs<T, K> p) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < ngroups;
       g += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t base = g;
#pragma unroll
    for (int s = 0; s < K; ++s) base = inject0(base, p.sorted[s]);
    C v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = a[base + p.off[c]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      C acc = CT<T>::make(0, 0);
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if (REAL)
          rmac(acc, p.m[r * D + c].x, v[c]);
        else
          cmac(acc, p.m[r * D + c], v[c]);
      }
      a[base + p.off[r]] = acc;
    }
  }
}

template <int K>
struct PermArgs {
  uint64_t off[1 << K];
  int sorted[K];
  int nmoved;
  unsigned char dst[1 << K];
  unsigned char src[1 << K];
};

template <typename T, int K>
__global__ void __launch_bounds__(256)
    k_perm(typename CT<T>::C *__restrict__ a, uint64_t ngroups,
           const __grid_constant__ PermArgs<K> p) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < ngroups;
       g += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t base = g;
#pragma unroll
    for (int s = 0; s < K; ++s) base = inject0(base, p.sorted[s]);
    C v[D];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < p.nmoved) v[j] = a[base + p.off[p.src[j]]];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < p.nmoved) a[base + p.off[p.dst[j]]] = v[j];
  }
}

constexpr int kMaxTables = 4;
constexpr int kMaxTableBits = 10;
constexpr int kMaxReq = 4;

struct DiagArgs {
  int ntables;
  int k[kMaxTables];
  int qubits[kMaxTables][kMaxTableBits];
  int start[kMaxTables];  // entry offset of each table
  // Ascending qubits that form at most two contiguous runs, lo1 .. lo1+n1-1
  // then lo2 .. lo2+k-n1-1 (lo1 = -1: any other set, gathered bit by bit).
  // A CPHASE chain's table -- a run of controls plus its target -- is one.
  int lo1[kMaxTables], n1[kMaxTables], lo2[kMaxTables];
  int total;              // total entries
  // Required qubits, ascending: every table holds them, and every entry with
  // one of them 0 is exactly 1 (a CPHASE's or CZ's two qubits, a CPHASE
  // chain's target).  Only amplitudes with all of them 1 can change, so the
  // kernels visit 2^(n - nreq) indices with those bits set.
  int nreq;
  int req[kMaxReq];
};

__device__ __forceinline__ int diag_index(const DiagArgs &p, int t, uint64_t i) {
  if (p.lo1[t] >= 0) {
    const int n1 = p.n1[t], n2 = p.k[t] - n1;
    const uint64_t a = (i >> p.lo1[t]) & ((1ull << n1) - 1ull);
    const uint64_t b = (i >> p.lo2[t]) & ((1ull << n2) - 1ull);
    return (int)(a | (b << n1));
  }
  int idx = 0;
  for (int j = 0; j < p.k[t]; ++j) idx |= (int)((i >> p.qubits[t][j]) & 1ull) << j;
  return idx;
}

// Index j of the visited subspace -> amplitude address: a 1 inserted at each
// required qubit (ascending).
__device__ __forceinline__ uint64_t diag_address(const DiagArgs &p, uint64_t j) {
  for (int r = 0; r < p.nreq; ++r) j = inject0(j, p.req[r]) | (1ull << p.req[r]);
  return j;
}

// The product of an amplitude's table entries is formed in double-float
// (dfc, cplx.h: FP32 pairs, ~47-bit significand) on the FP32 pipe; on this
// part the FP64 pipe runs at 1/64 of the FP32 rate.

// Product of an FP32 amplitude's table entries other than 1 ((1, 0) if none).
__device__ __forceinline__ float2 diag_phase_f32(const DiagArgs &p, const float2 *tab,
                                                 uint64_t i) {
  float2 ph = make_float2(1.f, 0.f);
  bool unit = true;
  for (int t = 0; t < p.ntables; ++t) {
    const float2 e = tab[p.start[t] + diag_index(p, t, i)];
    if (e.x == 1.f && e.y == 0.f) continue;
    ph = unit ? e : cmul(ph, e);
    unit = false;
  }
  return ph;
}

// FP32 states: tables and products in FP32.  Entries equal to 1 are
// skipped, and an amplitude whose phase is 1 is neither read nor written.
__global__ void __launch_bounds__(256)
    k_diag_tables_f32(float2 *__restrict__ a, uint64_t len, const float2 *__restrict__ tables,
                      const __grid_constant__ DiagArgs p) {
  extern __shared__ unsigned char smem_raw[];
  float2 *tab = reinterpret_cast<float2 *>(smem_raw);
  for (int j = threadIdx.x; j < p.total; j += blockDim.x) tab[j] = tables[j];
  __syncthreads();
  const uint64_t count = len >> p.nreq;
  if (p.nreq == 0 || p.req[0] > 0) {
    // Qubit 0 is not required: a thread takes the two amplitudes at i and
    // i + 1, one 16-byte load and store (a pair without a phase is skipped).
    float4 *a4 = reinterpret_cast<float4 *>(a);
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < count / 2;
         j += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t i = diag_address(p, 2 * j);
      const float2 ph0 = diag_phase_f32(p, tab, i), ph1 = diag_phase_f32(p, tab, i + 1);
      const bool u0 = ph0.x == 1.f && ph0.y == 0.f, u1 = ph1.x == 1.f && ph1.y == 0.f;
      if (u0 && u1) continue;
      const float4 v = a4[i >> 1];
      const float2 r0 = u0 ? make_float2(v.x, v.y) : cmul(make_float2(v.x, v.y), ph0);
      const float2 r1 = u1 ? make_float2(v.z, v.w) : cmul(make_float2(v.z, v.w), ph1);
      a4[i >> 1] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
    return;
  }
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < count;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = diag_address(p, j);
    const float2 ph = diag_phase_f32(p, tab, i);
    if (ph.x != 1.f || ph.y != 0.f) a[i] = cmul(a[i], ph);
  }
}

// FP64 states: the tables are held in shared memory as double-float pairs
// (converted once per CTA) and multiplied together in FP32 pairs; one FP64
// complex multiply applies the product.  An amplitude whose entries are all
// 1 is neither read nor written.
__global__ void __launch_bounds__(256)
    k_diag_tables_f64(double2 *__restrict__ a, uint64_t len, const double2 *__restrict__ tables,
                      const __grid_constant__ DiagArgs p) {
  extern __shared__ unsigned char smem_raw[];
  dfc *tab = reinterpret_cast<dfc *>(smem_raw);
  for (int j = threadIdx.x; j < p.total; j += blockDim.x) {
    const double2 e = tables[j];
    dfc d = df_from_double2_any(e);
    if (e.x == 1.0 && e.y == 0.0) d.rl = d.il = 0.f;  // exactly (1, 0): the skip test
    tab[j] = d;
  }
  __syncthreads();
  const uint64_t count = len >> p.nreq;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < count;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = diag_address(p, j);
    dfc ph;
    int nonunit = 0;
    for (int t = 0; t < p.ntables; ++t) {
      const dfc e = tab[p.start[t] + diag_index(p, t, i)];
      if (e.rh == 1.f && e.rl == 0.f && e.ih == 0.f && e.il == 0.f) continue;
      ph = nonunit ? df_cmul(ph, e) : e;
      ++nonunit;
    }
    if (!nonunit) continue;
    double2 f;
    if (nonunit == 1) {
      // a single entry: use its FP64 value exactly
      int t = 0;
      for (; t < p.ntables; ++t) {
        const dfc e = tab[p.start[t] + diag_index(p, t, i)];
        if (!(e.rh == 1.f && e.rl == 0.f && e.ih == 0.f && e.il == 0.f)) break;
      }
      f = tables[p.start[t] + diag_index(p, t, i)];
    } else {
      // float -> double by integer bit moves: only the two adds use the FP64 pipe
      f = make_double2(df_to_double(ph.rh, ph.rl), df_to_double(ph.ih, ph.il));
    }
    a[i] = cmul(a[i], f);
  }
}

// ---- host side ------------------------------------------------------------------

static void sorted_qubits(int k, const int *qubits, int *sorted) {
  std::copy(qubits, qubits + k, sorted);
  std::sort(sorted, sorted + k);
}

template <typename T, int K>
static int dense_impl(qvmg_state s, const int *qubits, const double *m, bool real) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  DenseArgs<T, K> p;
  for (int i = 0; i < D * D; ++i) p.m[i] = CT<T>::make((T)m[2 * i], (T)m[2 * i + 1]);
  for (int c = 0; c < D; ++c) {
    uint64_t o = 0;
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1ull << qubits[j];
    p.off[c] = o;
  }
  sorted_qubits(K, qubits, p.sorted);
  uint64_t ngroups = s->len >> K;
  int grid = grid_for(ngroups, 256);
  C *a = (C *)s->amps;
  if (real)
    k_dense<T, K, true><<<grid, 256, 0, s->stream>>>(a, ngroups, p);
  else
    k_dense<T, K, false><<<grid, 256, 0, s->stream>>>(a, ngroups, p);
  QVMG_CHECK_LAUNCH("k_dense");
  return QVMG_OK;
}

template <typename T>
static int dense_dispatch(qvmg_state s, int k, const int *qubits, const double *m, bool real) {
  switch (k) {
    case 1: return dense_impl<T, 1>(s, qubits, m, real);
    case 2: return dense_impl<T, 2>(s, qubits, m, real);
    case 3: return dense_impl<T, 3>(s, qubits, m, real);
    case 4: return dense_impl<T, 4>(s, qubits, m, real);
    case 5: return dense_impl<T, 5>(s, qubits, m, real);
  }
  return fail(QVMG_E_INVALID, "dense gate width must be 1..5");
}

template <typename T, int K>
static int perm_impl(qvmg_state s, const int *qubits, const int64_t *perm) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  PermArgs<K> p;
  for (int c = 0; c < D; ++c) {
    uint64_t o = 0;
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1ull << qubits[j];
    p.off[c] = o;
  }
  sorted_qubits(K, qubits, p.sorted);
  p.nmoved = 0;
  for (int j = 0; j < D; ++j) {
    if (perm[j] != j) {
      p.dst[p.nmoved] = (unsigned char)j;
      p.src[p.nmoved] = (unsigned char)perm[j];
      ++p.nmoved;
    }
  }
  if (p.nmoved == 0) return QVMG_OK;
  uint64_t ngroups = s->len >> K;
  k_perm<T, K><<<grid_for(ngroups, 256), 256, 0, s->stream>>>((C *)s->amps, ngroups, p);
  QVMG_CHECK_LAUNCH("k_perm");
  return QVMG_OK;
}

template <typename T>
static int perm_dispatch(qvmg_state s, int k, const int *qubits, const int64_t *perm) {
  switch (k) {
    case 1: return perm_impl<T, 1>(s, qubits, perm);
    case 2: return perm_impl<T, 2>(s, qubits, perm);
    case 3: return perm_impl<T, 3>(s, qubits, perm);
    case 4: return perm_impl<T, 4>(s, qubits, perm);
    case 5: return perm_impl<T, 5>(s, qubits, perm);
  }
  return fail(QVMG_E_INVALID, "permutation width must be 1..5");
}

int diag_required_bits(int ntables, const int *ks, const int *qubits, const double *tables,
                       int *req) {
  int nreq = 0;
  for (int j0 = 0; j0 < ks[0] && nreq < kMaxReq; ++j0) {
    const int q = qubits[j0];
    bool ok = true;
    int qoff = 0, eoff = 0;
    for (int t = 0; t < ntables && ok; ++t) {
      int pos = -1;
      for (int j = 0; j < ks[t]; ++j)
        if (qubits[qoff + j] == q) pos = j;
      if (pos < 0) ok = false;
      for (int e = 0; ok && e < (1 << ks[t]); ++e)
        if (!((e >> pos) & 1) && (tables[2 * (eoff + e)] != 1.0 || tables[2 * (eoff + e) + 1] != 0.0))
          ok = false;
      qoff += ks[t];
      eoff += 1 << ks[t];
    }
    if (ok) req[nreq++] = q;
  }
  std::sort(req, req + nreq);
  return nreq;
}

static int diag_args(int ntables, const int *ks, const int *qubits, DiagArgs &p) {
  std::memset(&p, 0, sizeof(p));
  p.ntables = ntables;
  int total = 0, qoff = 0;
  for (int t = 0; t < ntables; ++t) {
    p.k[t] = ks[t];
    for (int j = 0; j < ks[t]; ++j) p.qubits[t][j] = qubits[qoff + j];
    qoff += ks[t];
    p.start[t] = total;
    total += 1 << ks[t];
    // split the (ascending) qubits into contiguous runs; two runs at most
    // take the shift-and-mask path
    int runs = 1, n1 = ks[t];
    for (int j = 1; j < ks[t]; ++j) {
      if (p.qubits[t][j] <= p.qubits[t][j - 1]) runs = 3;  // not ascending
      else if (p.qubits[t][j] != p.qubits[t][j - 1] + 1) {
        if (runs == 1) n1 = j;
        ++runs;
      }
    }
    if (runs <= 2) {
      p.lo1[t] = p.qubits[t][0];
      p.n1[t] = n1;
      p.lo2[t] = n1 < ks[t] ? p.qubits[t][n1] : 0;
    } else {
      p.lo1[t] = -1;
    }
  }
  p.total = total;
  return total;
}

template <typename T>
static int diag_dev_impl(qvmg_state s, const DiagArgs &p, const void *dtables) {
  using C = typename CT<T>::C;
  if constexpr (sizeof(T) == 8) {
    const size_t smem = p.total * sizeof(dfc);
    k_diag_tables_f64<<<grid_for(s->len, 256), 256, smem, s->stream>>>(
        (double2 *)s->amps, s->len, (const double2 *)dtables, p);
  } else {
    const size_t smem = p.total * sizeof(C);
    k_diag_tables_f32<<<grid_for(s->len, 256), 256, smem, s->stream>>>(
        (float2 *)s->amps, s->len, (const float2 *)dtables, p);
  }
  QVMG_CHECK_LAUNCH("k_diag_tables");
  return QVMG_OK;
}

template <typename T>
static int diag_tables_impl(qvmg_state s, int ntables, const int *ks, const int *qubits,
                            const double *tables) {
  using C = typename CT<T>::C;
  DiagArgs p;
  int total = diag_args(ntables, ks, qubits, p);
  p.nreq = diag_required_bits(ntables, ks, qubits, tables, p.req);
  std::vector<C> host(total);
  for (int i = 0; i < total; ++i) host[i] = CT<T>::make((T)tables[2 * i], (T)tables[2 * i + 1]);
  int rc = ensure_dvec(s, total * sizeof(C));
  if (rc) return rc;
  QVMG_CUDA(cudaMemcpyAsync(s->dvec, host.data(), total * sizeof(C), cudaMemcpyHostToDevice,
                            s->stream));
  // The host vector dies at return: make sure the copy has consumed it.
  QVMG_CUDA(cudaStreamSynchronize(s->stream));
  return diag_dev_impl<T>(s, p, s->dvec);
}

// Attribute setup for the large-smem diagonal kernel.
static int diag_attr() {
  static std::once_flag flag;
  static cudaError_t err = cudaSuccess;
  QVMG_CUDA(once(flag, err, [] {
    const int bytes = kMaxTables * (1 << kMaxTableBits) * 16;
    cudaError_t e = cudaFuncSetAttribute(k_diag_tables_f64,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_diag_tables_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               bytes);
    return e;
  }));
  return QVMG_OK;
}

int launch_diag_tables(qvmg_state s, int ntables, const int *ks, const int *qubits,
                       const double *tables) {
  if (ntables < 1 || ntables > kMaxTables)
    return fail(QVMG_E_INVALID, "diagonal pass needs 1..4 tables");
  for (int t = 0; t < ntables; ++t)
    if (ks[t] < 1 || ks[t] > kMaxTableBits)
      return fail(QVMG_E_INVALID, "diagonal table width must be 1..10");
  int rc = diag_attr();
  if (rc) return rc;
  if (s->prec == QVMG_FP64) return diag_tables_impl<double>(s, ntables, ks, qubits, tables);
  return diag_tables_impl<float>(s, ntables, ks, qubits, tables);
}

int launch_diag_dev(qvmg_state s, int ntables, const int *ks, const int *qubits,
                    const void *dtables, int nreq, const int *req) {
  if (ntables < 1 || ntables > kMaxTables)
    return fail(QVMG_E_INVALID, "diagonal pass needs 1..4 tables");
  if (nreq < 0 || nreq > kMaxReq) return fail(QVMG_E_INVALID, "too many required qubits");
  int rc = diag_attr();
  if (rc) return rc;
  DiagArgs p;
  diag_args(ntables, ks, qubits, p);
  p.nreq = nreq;
  for (int r = 0; r < nreq; ++r) p.req[r] = req[r];
  if (s->prec == QVMG_FP64) return diag_dev_impl<double>(s, p, dtables);
  return diag_dev_impl<float>(s, p, dtables);
}

int launch_dense(qvmg_state s, int k, const int *qubits, const double *m) {
  bool real = true;
  for (int i = 0; i < (1 << (2 * k)); ++i)
    if (m[2 * i + 1] != 0.0) { real = false; break; }
  if (s->prec == QVMG_FP64) return dense_dispatch<double>(s, k, qubits, m, real);
  return dense_dispatch<float>(s, k, qubits, m, real);
}

int launch_permutation(qvmg_state s, int k, const int *qubits, const int64_t *perm) {
  if (s->prec == QVMG_FP64) return perm_dispatch<double>(s, k, qubits, perm);
  return perm_dispatch<float>(s, k, qubits, perm);
}

int launch_diagonal(qvmg_state s, int k, const int *qubits, const double *diag) {
  return launch_diag_tables(s, 1, &k, qubits, diag);
}

// Matrix classification: the compile-gate specialisations of constant
// matrices (src/compile-gate.lisp:113-209, :259-309).
bool matrix_is_diagonal(int k, const double *m) {
  int d = 1 << k;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c)
      if (r != c && (m[2 * (r * d + c)] != 0.0 || m[2 * (r * d + c) + 1] != 0.0)) return false;
  return true;
}

bool matrix_is_permutation(int k, const double *m, int64_t *perm) {
  int d = 1 << k;
  std::vector<int> seen(d, 0);
  for (int r = 0; r < d; ++r) {
    int one = -1;
    for (int c = 0; c < d; ++c) {
      double re = m[2 * (r * d + c)], im = m[2 * (r * d + c) + 1];
      if (re == 1.0 && im == 0.0) {
        if (one >= 0) return false;
        one = c;
      } else if (re != 0.0 || im != 0.0) {
        return false;
      }
    }
    if (one < 0 || seen[one]) return false;
    seen[one] = 1;
    perm[r] = one;
  }
  return true;
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

int qvmg_apply_dense(qvmg_state s, int k, const int *qubits, const double *matrix) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubits(s, k, qubits, QVMG_MAX_GATE_QUBITS))) return rc;
  if (!matrix) return fail(QVMG_E_INVALID, "null matrix");
  int64_t perm[32];
  if (matrix_is_permutation(k, matrix, perm)) return launch_permutation(s, k, qubits, perm);
  if (matrix_is_diagonal(k, matrix)) {
    std::vector<double> diag(2 << k);
    int d = 1 << k;
    for (int j = 0; j < d; ++j) {
      diag[2 * j] = matrix[2 * (j * d + j)];
      diag[2 * j + 1] = matrix[2 * (j * d + j) + 1];
    }
    return launch_diagonal(s, k, qubits, diag.data());
  }
  return launch_dense(s, k, qubits, matrix);
}

int qvmg_apply_permutation(qvmg_state s, int k, const int *qubits, const int64_t *perm) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubits(s, k, qubits, QVMG_MAX_GATE_QUBITS))) return rc;
  if (!perm) return fail(QVMG_E_INVALID, "null permutation");
  int d = 1 << k;
  std::vector<int> seen(d, 0);
  for (int j = 0; j < d; ++j) {
    if (perm[j] < 0 || perm[j] >= d || seen[perm[j]])
      return fail(QVMG_E_INVALID, "not a permutation of 0..2^k-1");
    seen[perm[j]] = 1;
  }
  return launch_permutation(s, k, qubits, perm);
}

int qvmg_apply_diagonal(qvmg_state s, int k, const int *qubits, const double *diag) {
  int rc = check_state(s);
  if (rc) return rc;
  if ((rc = check_qubits(s, k, qubits, QVMG_MAX_DIAG_QUBITS))) return rc;
  if (!diag) return fail(QVMG_E_INVALID, "null diagonal");
  return launch_diagonal(s, k, qubits, diag);
}

}  // extern "C"
