// batch.cu -- batched QAOA MaxCut instances in one persistent launch.
//
// The reference runs one QVM per request and re-runs the program per trial
// (app/src/api/multishot.lisp:87-101; examples/qaoa.lisp:118-183 samples
// each QAOA wavefunction with sample-wavefunction-multiple-times).  Here a
// batch of uneven instances (different qubit counts, graphs and angles) runs
// in one persistent kernel: each CTA takes the next instance from a device
// work queue (an atomic counter, instances sorted largest first) and runs
// the whole circuit for it:
//   H on all qubits                 -> amplitudes start at 2^(-n/2)
//   per layer l: ZZ(gamma_l) on every edge, i.e. the diagonal
//                exp(-i gamma_l (m - 2 cut(x)) / 2), then RX(2 beta_l) on
//                every qubit
//   <H_C> = sum_x |a_x|^2 cut(x)   (FP64 accumulation)
//   shots: a two-level CDF (128-amplitude sub-block sums, FP64 prefix)
//          searched per draw by one warp, smallest x with C(x) >= draw.
// States of <= 13 qubits live in shared memory for the whole circuit.
// Larger ones stay in HBM and are swept in tile passes of two kinds:
// contiguous tiles (qubits 0..12) and rows of 2^(26-n) amplitudes holding the
// high qubits.  The kinds alternate, and each pass finishes the previous
// layer's RX on the qubits the previous pass lacked, then applies the next
// layer's phase and its RX on all 13 tile qubits: p layers take p + 1 passes
// (two per layer before: 4 layers at 22 qubits read and wrote the state 8
// times, now 5).  The first pass makes its tiles from the uniform state and
// writes every amplitude's cut value as one byte beside the state; later
// passes load those bytes with their tiles for the phase, and a last
// contiguous pass takes <H_C> and the CDF sub-block sums from its tiles.
// (Streaming tiles through two buffers per CTA was measured too: 13-qubit
// tiles leave one CTA per SM, 143 -> 199 ms for the 4096-instance batch;
// 12-qubit tiles keep three CTAs per SM but give 32-byte rows in the second
// pass at 22 qubits, 140 -> 166 ms.)  Amplitudes are complex FP32; the phase
// table and RX coefficients are computed in FP64.  The first pass takes each
// amplitude's cut from a per-instance table of the edges inside the low 13
// bits, a constant per row for the edges inside the high bits and popcounts
// over the cross edges (cut_split).  RX runs in register sweeps of up to
// four qubits (each thread holds a group of 16 amplitudes), a layer's phase
// folded into the first sweep of its RX.
// All spin-free: the queue is a plain atomicAdd, no CTA waits on another.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "cplx.h"
#include "internal.h"

namespace qvmg {

constexpr int kQaoaTileBits = 13;
constexpr int kQaoaThreads = 256;
constexpr int kQaoaMaxEdges = 64;
constexpr int kQaoaMaxLayers = 16;
constexpr int kQaoaSubBits = 7;  // 128-amplitude CDF sub-blocks

struct QaoaInst {
  unsigned long long state_off;  // float2 offset of the state
  unsigned long long sub_off;    // double offset of the CDF sub-block sums
  unsigned long long cut_off;    // byte offset of the cut values (states in HBM)
  int n;
  int nedges;
  int edge_off;   // into edges (pairs)
  int param_off;  // into gammas / betas (p values)
  int id;         // caller's instance index
  int pad;
};

struct QaoaArgs {
  int ninst;
  int p;
  int nshots;
  int pad;
  const QaoaInst *inst;
  const unsigned char *edges;  // pairs (u, v)
  const double *gammas;
  const double *betas;
  float2 *states;
  double *subs;
  unsigned char *cuts;        // one cut byte per amplitude of each state in HBM
  const double *draws;        // ninst * nshots, indexed by instance id
  double *expect;             // ninst
  unsigned int *shots;        // ninst * nshots
  unsigned int *counter;      // work queue head
};

__device__ __forceinline__ int cut_value(unsigned long long x, const unsigned char *e, int m) {
  int c = 0;
  for (int i = 0; i < m; ++i) c += (int)(((x >> e[2 * i]) ^ (x >> e[2 * i + 1])) & 1ull);
  return c;
}

// The cut of x split by where each edge's endpoints lie against the 13-bit
// tile (x = h << 13 | j): edges inside the low bits give a per-instance byte
// table cl[j]; edges inside the high bits a constant per h; an edge between a
// low qubit u and a high qubit v counts (j_u xor h_v).  The cross edges are
// spread over up to kCutSlots slots, each low qubit at most once per slot, so
// that their sum is popc((j ^ F_k) & M_k) over the slots: M_k the slot's low
// qubits, F_k those whose high partner is 1 in h.
constexpr int kCutSlots = 4;
constexpr unsigned char kSlotLow = 255, kSlotHigh = 254;

// F_k and the high-high count for high part h: warp-collective (all 32
// lanes), every lane gets the results.
__device__ __forceinline__ void cut_row(unsigned long long h, const unsigned char *e,
                                        const unsigned char *slot, int m, unsigned *F, int &ch) {
  const int lane = threadIdx.x & 31;
  unsigned f0 = 0, f1 = 0, f2 = 0, f3 = 0;
  int c = 0;
  for (int i = lane; i < m; i += 32) {
    const int u = e[2 * i], v = e[2 * i + 1], sl = slot[i];
    if (sl == kSlotHigh) {
      c += (int)(((h >> (u - kQaoaTileBits)) ^ (h >> (v - kQaoaTileBits))) & 1ull);
    } else if (sl < kCutSlots) {
      const int lo = u < v ? u : v, hi = u < v ? v : u;
      const unsigned bit = (unsigned)((h >> (hi - kQaoaTileBits)) & 1ull) << lo;
      if (sl == 0) f0 |= bit;
      else if (sl == 1) f1 |= bit;
      else if (sl == 2) f2 |= bit;
      else f3 |= bit;
    }
  }
  F[0] = __reduce_or_sync(0xffffffffu, f0);
  F[1] = __reduce_or_sync(0xffffffffu, f1);
  F[2] = __reduce_or_sync(0xffffffffu, f2);
  F[3] = __reduce_or_sync(0xffffffffu, f3);
  ch = __reduce_add_sync(0xffffffffu, c);
}

__device__ __forceinline__ int cut_split(unsigned j, const unsigned char *cl, const unsigned *F,
                                         const unsigned *M, int ch) {
  return (int)cl[j] + ch + __popc((j ^ F[0]) & M[0]) + __popc((j ^ F[1]) & M[1]) +
         __popc((j ^ F[2]) & M[2]) + __popc((j ^ F[3]) & M[3]);
}

// RX(2 beta) = [[c, -is], [-is, c]] with its larger coefficient factored
// out: c (I - i t X), t = tan(beta), when |c| >= |s| (KFORM false), else
// s (k I - i X), k = cot(beta).  The factor (c^n or s^n for the n qubits)
// goes into the layer's phase table, so a pair costs four FMAs.  Symmetric
// in the two basis states, so the pair's order does not matter.
template <bool KFORM>
__device__ __forceinline__ void rx_pair(float2 &a, float2 &b, float w) {
  const float2 x = a, y = b;
  if constexpr (KFORM) {
    a = make_float2(fmaf(w, x.x, y.y), fmaf(w, x.y, -y.x));
    b = make_float2(fmaf(w, y.x, x.y), fmaf(w, y.y, -x.x));
  } else {
    a = make_float2(fmaf(w, y.y, x.x), fmaf(-w, y.x, x.y));
    b = make_float2(fmaf(w, x.y, y.x), fmaf(-w, x.x, y.y));
  }
}

// A tile's phases: the layer's table indexed by each amplitude's cut value,
// held as one byte per tile element (the low-edge table of a resident state,
// or the cut bytes loaded beside the tile).
struct PhaseSrc {
  const float2 *phase;
  const unsigned char *cut;
  __device__ __forceinline__ float2 at(unsigned j) const { return phase[cut[j]]; }
};

// One register sweep of a shared-memory tile of 2^tb amplitudes: every
// thread takes groups of 2^R amplitudes spanning tile bits first ..
// first+R-1, multiplies them by the layer's phase first when PHASE, and
// applies RX(2 beta) on all R bits in registers.  A sweep that starts at
// tile bit 0 spans consecutive amplitudes: each lane then visits its group's
// members in an order XORed with its lane index, so that the lanes of a warp
// hit distinct banks; RX is symmetric, so the butterflies pair the same
// registers whatever the order.
template <int R, bool PHASE, bool KFORM>
__device__ __forceinline__ void rx_sweep(float2 *tile, int tb, int first, float w,
                                         const PhaseSrc &ph) {
  constexpr int G = 1 << R;
  const unsigned rot = first == 0 ? (threadIdx.x & (unsigned)(G - 1)) : 0u;
  const unsigned ngroups = 1u << (tb - R);
  const unsigned lowmask = (1u << first) - 1u;
  for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x) {
    const unsigned b = ((g >> first) << (first + R)) | (g & lowmask);
    float2 v[G];
#pragma unroll
    for (int r = 0; r < G; ++r) {
      const unsigned j = b | ((r ^ rot) << first);
      v[r] = tile[j];
      if constexpr (PHASE) v[r] = cmul(v[r], ph.at(j));
    }
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int r = 0; r < G; ++r)
        if (!((r >> i) & 1)) rx_pair<KFORM>(v[r], v[r | (1 << i)], w);
#pragma unroll
    for (int r = 0; r < G; ++r) tile[b | ((r ^ rot) << first)] = v[r];
  }
}

// RX on tile bits first .. first+count-1 in sweeps of up to 4 bits, the
// phase folded into the first sweep when `phase`.
template <bool KFORM>
__device__ __forceinline__ void tile_rx_run_f(float2 *tile, int tb, int first, int count, float w,
                                              bool phase, const PhaseSrc &ph) {
  for (int q = 0; q < count; q += 4) {
    const int r = count - q < 4 ? count - q : 4;
    const bool ph_now = phase && q == 0;
    switch (r * 2 + (ph_now ? 1 : 0)) {
      case 2: rx_sweep<1, false, KFORM>(tile, tb, first + q, w, ph); break;
      case 3: rx_sweep<1, true, KFORM>(tile, tb, first + q, w, ph); break;
      case 4: rx_sweep<2, false, KFORM>(tile, tb, first + q, w, ph); break;
      case 5: rx_sweep<2, true, KFORM>(tile, tb, first + q, w, ph); break;
      case 6: rx_sweep<3, false, KFORM>(tile, tb, first + q, w, ph); break;
      case 7: rx_sweep<3, true, KFORM>(tile, tb, first + q, w, ph); break;
      case 8: rx_sweep<4, false, KFORM>(tile, tb, first + q, w, ph); break;
      default: rx_sweep<4, true, KFORM>(tile, tb, first + q, w, ph); break;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void tile_rx_run(float2 *tile, int tb, int first, int count, float w,
                                            bool kform, bool phase, const PhaseSrc &ph) {
  if (kform) tile_rx_run_f<true>(tile, tb, first, count, w, phase, ph);
  else tile_rx_run_f<false>(tile, tb, first, count, w, phase, ph);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double prob_d(float2 v) {
  return (double)v.x * (double)v.x + (double)v.y * (double)v.y;
}

// RX(2 beta) in the factored form of rx_pair: returns the coefficient w,
// whether the sine was factored out, and the factor (cos or sin beta).
__device__ __forceinline__ float rx_coef(double beta, bool &kform, double &factor) {
  double rs, rc;
  sincos(beta, &rs, &rc);
  kform = fabs(rs) > fabs(rc);
  factor = kform ? rs : rc;
  return (float)(kform ? rc / rs : rs / rc);
}

// A layer's phase table exp(-i gamma (m - 2c) / 2), c = 0..m, scaled by the
// RX factor of all n qubits (rx_coef); the CTA's threads share the entries.
__device__ __forceinline__ void phase_table(float2 *phase, double gamma, double factor, int n,
                                            int m) {
  const double fac = pow(factor, (double)n);
  for (int c = threadIdx.x; c <= m; c += blockDim.x) {
    double sn, cs;
    sincos(-gamma * (double)(m - 2 * c) * 0.5, &sn, &cs);
    phase[c] = make_float2((float)(fac * cs), (float)(fac * sn));
  }
}

__global__ void __launch_bounds__(kQaoaThreads, 3) k_qaoa_batch(const __grid_constant__ QaoaArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *tile = reinterpret_cast<float2 *>(smem);                     // 2^13
  // 2^13 cut bytes (the low-edge table, or a tile's cut values), 16-byte aligned
  unsigned char *cl = smem + (8u << kQaoaTileBits);
  float2 *phase = reinterpret_cast<float2 *>(cl + (1u << kQaoaTileBits));  // kQaoaMaxEdges+1
  unsigned char *edges = reinterpret_cast<unsigned char *>(phase + kQaoaMaxEdges + 1);
  __shared__ double red[kQaoaThreads / 32];
  __shared__ int s_inst;
  __shared__ unsigned char s_slot[kQaoaMaxEdges];
  __shared__ unsigned s_M[kCutSlots];
  __shared__ int s_split;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_inst = (int)atomicAdd(A.counter, 1u);
    __syncthreads();
    const int k = s_inst;
    if (k >= A.ninst) break;
    const QaoaInst I = A.inst[k];
    const int n = I.n, m = I.nedges;
    float2 *psi = A.states + I.state_off;
    for (int i = threadIdx.x; i < 2 * m; i += blockDim.x) edges[i] = A.edges[2 * I.edge_off + i];
    __syncthreads();
    if (threadIdx.x == 0) {
      // edge classes and cross-edge slots (the split cut; more than
      // kCutSlots cross edges on one low qubit: the edge loop instead)
      unsigned char cnt[kQaoaTileBits] = {};
      unsigned M[kCutSlots] = {};
      int ok = 1;
      for (int i = 0; i < m; ++i) {
        const int u = edges[2 * i], v = edges[2 * i + 1];
        const bool ul = u < kQaoaTileBits, vl = v < kQaoaTileBits;
        unsigned char sl = ul && vl ? kSlotLow : (!ul && !vl ? kSlotHigh : 0);
        if (ul != vl) {
          const int lo = ul ? u : v;
          const int kk = cnt[lo]++;
          if (kk >= kCutSlots) ok = 0;
          else M[kk] |= 1u << lo;
          sl = (unsigned char)(kk < kCutSlots ? kk : kSlotLow);
        }
        s_slot[i] = sl;
      }
      for (int k = 0; k < kCutSlots; ++k) s_M[k] = M[k];
      s_split = ok;
    }
    __syncthreads();
    const bool split = s_split != 0;
    if (split) {
      const unsigned nlow = 1u << (n < kQaoaTileBits ? n : kQaoaTileBits);
      for (unsigned j = threadIdx.x; j < nlow; j += blockDim.x) {
        int c = 0;
        for (int i = 0; i < m; ++i)
          if (s_slot[i] == kSlotLow) c += (int)(((j >> edges[2 * i]) ^ (j >> edges[2 * i + 1])) & 1u);
        cl[j] = (unsigned char)c;
      }
    }
    const unsigned long long len = 1ull << n;
    const float amp0 = (float)(1.0 / sqrt((double)len));
    const bool resident = n <= kQaoaTileBits;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int sbits = n < kQaoaSubBits ? n : kQaoaSubBits;
    const unsigned long long nsub = len >> sbits;
    double *sub = A.subs + I.sub_off;
    // every amplitude's cut value: the low-edge table of a resident state,
    // the bytes beside a state in HBM
    unsigned char *cuts = resident ? cl : A.cuts + I.cut_off;
    double ex = 0.0;      // this lane's share of <H_C>
    bool summed = false;  // sub-block sums and <H_C> taken in the last tile pass
    const PhaseSrc ph{phase, cl};
    if (resident) {
      // H on all qubits, then every layer on the state held in the tile
      for (unsigned x = threadIdx.x; x < len; x += blockDim.x) tile[x] = make_float2(amp0, 0.f);
      for (int l = 0; l < A.p; ++l) {
        __syncthreads();
        bool kf;
        double f1;
        const float w = rx_coef(A.betas[I.param_off + l], kf, f1);
        phase_table(phase, A.gammas[I.param_off + l], f1, n, m);
        __syncthreads();
        tile_rx_run(tile, n, 0, n, w, kf, true, ph);
      }
      __syncthreads();
      for (unsigned x = threadIdx.x; x < len; x += blockDim.x) psi[x] = tile[x];
      __syncthreads();
    } else {
      // Tile passes over the state in HBM.  Type A passes (even) take
      // contiguous tiles, qubits 0..12; type B passes (odd) take rows of
      // 2^Lb amplitudes, qubits 0..Lb-1 and the high qubits 13..n-1.  Pass i
      // finishes layer i-1's RX on the tile bits Lb..12 (the qubits the
      // previous pass lacked), then applies layer i's phase and its RX on all
      // 13 tile qubits: p layers take p + 1 passes.  Pass 0 makes its tiles
      // from the uniform state and writes each amplitude's cut value (one
      // byte) beside the state; later passes load those bytes with the tile,
      // into the low-edge table's space.
      const int tb = kQaoaTileBits, hb = n - tb, Lb = tb - hb;  // n <= 26 keeps Lb >= 0
      const unsigned long long ntiles = len >> tb;
      const unsigned lomask = (1u << Lb) - 1u;
      const unsigned M[kCutSlots] = {s_M[0], s_M[1], s_M[2], s_M[3]};
      bool kf_prev = false;
      float w_prev = 0.f;
      for (int pass = 0; pass <= A.p; ++pass) {
        const bool rows = (pass & 1) != 0;
        const bool last = pass == A.p;
        bool kf = false;
        float w = 0.f;
        __syncthreads();  // the previous pass's phase table is no longer read
        if (!last) {
          double f1;
          w = rx_coef(A.betas[I.param_off + pass], kf, f1);
          phase_table(phase, A.gammas[I.param_off + pass], f1, n, m);
        }
        for (unsigned long long cidx = 0; cidx < ntiles; ++cidx) {
          __syncthreads();
          if (pass == 0) {
            // uniform amplitudes times layer 0's phase; the cut bytes go out
            const unsigned long long base = cidx << tb;
            unsigned F[kCutSlots] = {0u, 0u, 0u, 0u};
            int ch = 0;
            if (split) cut_row(cidx, edges, s_slot, m, F, ch);
            for (unsigned q = threadIdx.x; q < (1u << tb) / 4; q += blockDim.x) {
              unsigned word = 0;
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const unsigned j = 4 * q + e;
                const int cx = split ? cut_split(j, cl, F, M, ch) : cut_value(base + j, edges, m);
                const float2 f = phase[cx];
                tile[j] = make_float2(amp0 * f.x, amp0 * f.y);
                word |= (unsigned)cx << (8 * e);
              }
              reinterpret_cast<unsigned *>(cuts + base)[q] = word;
            }
          } else if (!rows) {
            // every 16-byte load of the tile and its cut bytes in flight at once
            const unsigned long long base = cidx << tb;
            for (unsigned j = threadIdx.x; j < (1u << tb) / 2; j += blockDim.x)
              cp_async16(reinterpret_cast<float4 *>(tile) + j,
                         reinterpret_cast<const float4 *>(psi + base) + j);
            for (unsigned j = threadIdx.x; j < (1u << tb) / 16; j += blockDim.x)
              cp_async16(cl + 16 * j, cuts + base + 16 * j);
            cp_async_wait_all();
          } else {
            if (Lb >= 1) {
              // rows of >= 2 amplitudes: 16-byte asynchronous loads
              for (unsigned j = 2 * threadIdx.x; j < (1u << tb); j += 2 * blockDim.x) {
                const unsigned long long h = j >> Lb, lo = j & lomask;
                cp_async16(tile + j, psi + ((h << tb) | (cidx << Lb) | lo));
              }
            } else {
              for (unsigned j = threadIdx.x; j < (1u << tb); j += blockDim.x)
                tile[j] = psi[((unsigned long long)j << tb) | cidx];
            }
            if (Lb >= 4) {
              for (unsigned j = 16 * threadIdx.x; j < (1u << tb); j += 16 * blockDim.x) {
                const unsigned long long h = j >> Lb, lo = j & lomask;
                cp_async16(cl + j, cuts + ((h << tb) | (cidx << Lb) | lo));
              }
            } else {
              for (unsigned j = threadIdx.x; j < (1u << tb); j += blockDim.x) {
                const unsigned long long h = j >> Lb, lo = j & lomask;
                cl[j] = cuts[(h << tb) | (cidx << Lb) | lo];
              }
            }
            cp_async_wait_all();
          }
          __syncthreads();
          if (pass > 0) tile_rx_run(tile, tb, Lb, hb, w_prev, kf_prev, false, ph);
          if (!last) {
            tile_rx_run(tile, tb, 0, tb, w, kf, pass > 0, ph);
          } else if (!rows) {
            // the last pass holds contiguous tiles: their 128-amplitude
            // sub-block sums and <H_C> terms, one warp per sub-block
            const unsigned long long s0 = cidx << (tb - kQaoaSubBits);
            for (unsigned sb = warp; sb < (1u << (tb - kQaoaSubBits)); sb += nwarps) {
              float hi = 0.f, lo = 0.f, exf = 0.f;
              for (unsigned j = lane; j < (1u << kQaoaSubBits); j += 32) {
                const unsigned t = (sb << kQaoaSubBits) + j;
                const float2 v = tile[t];
                df_add_prob(hi, lo, v);  // exact squares for the CDF
                exf = fmaf(fmaf(v.x, v.x, v.y * v.y), (float)cl[t], exf);
              }
              const double acc = warp_sum_d((double)hi + (double)lo);
              ex += (double)exf;
              if (lane == 0) sub[s0 + sb] = acc;
            }
          }
          if (!rows) {
            const unsigned long long base = cidx << tb;
            for (unsigned j = threadIdx.x; j < (1u << tb) / 2; j += blockDim.x)
              reinterpret_cast<float4 *>(psi + base)[j] = reinterpret_cast<const float4 *>(tile)[j];
          } else if (Lb >= 1) {
            for (unsigned j = 2 * threadIdx.x; j < (1u << tb); j += 2 * blockDim.x) {
              const unsigned long long h = j >> Lb, lo = j & lomask;
              *reinterpret_cast<float4 *>(psi + ((h << tb) | (cidx << Lb) | lo)) =
                  *reinterpret_cast<const float4 *>(tile + j);
            }
          } else {
            for (unsigned j = threadIdx.x; j < (1u << tb); j += blockDim.x)
              psi[((unsigned long long)j << tb) | cidx] = tile[j];
          }
        }
        w_prev = w;
        kf_prev = kf;
      }
      summed = (A.p & 1) == 0;
      __syncthreads();
    }
    if (!summed) {
      // expectation and 128-amplitude sub-block sums (one warp per sub-block)
      for (unsigned long long sb = warp; sb < nsub; sb += nwarps) {
        float hi = 0.f, lo = 0.f, exf = 0.f;
        for (unsigned j = lane; j < (1u << sbits); j += 32) {
          const unsigned long long x = (sb << sbits) + j;
          const float2 v = psi[x];
          df_add_prob(hi, lo, v);  // exact squares for the CDF
          exf = fmaf(fmaf(v.x, v.x, v.y * v.y), (float)cuts[x], exf);
        }
        const double acc = warp_sum_d((double)hi + (double)lo);
        ex += (double)exf;
        if (lane == 0) sub[sb] = acc;
      }
    }
    ex = warp_sum_d(ex);
    if (lane == 0) red[warp] = ex;
    __syncthreads();
    if (threadIdx.x == 0) {
      double e = 0.0;
      for (int w = 0; w < nwarps; ++w) e += red[w];
      A.expect[I.id] = e;
    }
    // inclusive prefix over the sub-block sums: per-thread chunks, then a
    // scan of the chunk totals in shared memory (the tile is free now)
    {
      double *tot = reinterpret_cast<double *>(tile);
      const unsigned long long per = (nsub + blockDim.x - 1) / blockDim.x;
      const unsigned long long a0 = threadIdx.x * per;
      const unsigned long long a1 = min(nsub, a0 + per);
      double s = 0.0;
      for (unsigned long long i = a0; i < a1; ++i) s += sub[i];
      tot[threadIdx.x] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        double r = 0.0;
        for (unsigned w = 0; w < blockDim.x; ++w) {
          double v = tot[w];
          tot[w] = r;
          r += v;
        }
      }
      __syncthreads();
      double r = tot[threadIdx.x];
      for (unsigned long long i = a0; i < a1; ++i) {
        r += sub[i];
        sub[i] = r;
      }
    }
    __syncthreads();
    // shots: smallest x with C(x) >= draw (src/measurement.lisp:246-288), len-1 if none
    for (int t = warp; t < A.nshots; t += nwarps) {
      // renormalised FP32 distribution, as in qvmg_sample
      const double p = A.draws[(unsigned long long)I.id * A.nshots + t] * sub[nsub - 1];
      unsigned long long lo = 0, hi = nsub;
      while (lo < hi) {
        unsigned long long mid = (lo + hi) >> 1;
        if (sub[mid] >= p) hi = mid; else lo = mid + 1;
      }
      unsigned int res = (unsigned int)(len - 1);
      if (lo < nsub) {
        double run = lo ? sub[lo - 1] : 0.0;
        res = (unsigned int)(((lo + 1) << sbits) - 1);
        for (unsigned c0 = 0; c0 < (1u << sbits); c0 += 32) {
          const bool valid = c0 + lane < (1u << sbits);
          double pr = valid ? prob_d(psi[(lo << sbits) + c0 + lane]) : 0.0;
          double sc = pr;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            double y = __shfl_up_sync(0xffffffffu, sc, o);
            if (lane >= o) sc += y;
          }
          unsigned msk = __ballot_sync(0xffffffffu, valid && run + sc >= p);
          if (msk) {
            res = (unsigned int)((lo << sbits) + c0 + (__ffs(msk) - 1));
            break;
          }
          run += __shfl_sync(0xffffffffu, sc, 31);
        }
      }
      if (lane == 0) A.shots[(unsigned long long)I.id * A.nshots + t] = res;
    }
  }
}

}  // namespace qvmg

struct qvmg_qaoa_s {
  int ninst = 0, p = 0;
  std::vector<int> n;                // per caller instance
  std::vector<unsigned long long> state_off;
  qvmg::QaoaArgs args{};
  void *dbuf = nullptr;              // instances, edges, params
  float2 *states = nullptr;
  double *subs = nullptr;
  unsigned char *cuts = nullptr;
  double *draws = nullptr;
  double *expect = nullptr;
  unsigned int *shots = nullptr;
  unsigned int *counter = nullptr;
  int nshots_cap = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_shots = -1;
  uint64_t bytes = 0;
};

using namespace qvmg;

static void qaoa_release(qvmg_qaoa_batch b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->dbuf);
  cudaFree(b->states);
  cudaFree(b->subs);
  cudaFree(b->cuts);
  cudaFree(b->draws);
  cudaFree(b->expect);
  cudaFree(b->shots);
  cudaFree(b->counter);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" {

int qvmg_qaoa_batch_create(int ninst, const int *nqubits, const int *nedges, const int *edges,
                           int p, const double *gammas, const double *betas,
                           qvmg_qaoa_batch *out) {
  if (!out) return fail(QVMG_E_INVALID, "null output handle");
  *out = nullptr;
  if (ninst < 1 || !nqubits || !nedges || !edges || !gammas || !betas)
    return fail(QVMG_E_INVALID, "empty batch or null array");
  if (p < 1 || p > kQaoaMaxLayers) return fail(QVMG_E_INVALID, "QAOA depth must be 1..16");
  std::vector<QaoaInst> inst(ninst);
  std::vector<unsigned char> e8;
  unsigned long long soff = 0, uoff = 0, coff = 0;
  int eoff = 0;
  for (int i = 0; i < ninst; ++i) {
    int n = nqubits[i];
    if (n < 2 || n > 26) return fail(QVMG_E_INVALID, "instance qubit count must be 2..26");
    if (nedges[i] < 0 || nedges[i] > kQaoaMaxEdges)
      return fail(QVMG_E_INVALID, "instance edge count must be 0..64");
    inst[i].n = n;
    inst[i].nedges = nedges[i];
    inst[i].edge_off = eoff;
    inst[i].param_off = i * p;
    inst[i].id = i;
    for (int j = 0; j < nedges[i]; ++j) {
      int u = edges[2 * (eoff + j)], v = edges[2 * (eoff + j) + 1];
      if (u < 0 || v < 0 || u >= n || v >= n || u == v)
        return fail(QVMG_E_INVALID, "edge (" + std::to_string(u) + "," + std::to_string(v) +
                                        ") invalid for instance " + std::to_string(i));
      e8.push_back((unsigned char)u);
      e8.push_back((unsigned char)v);
    }
    eoff += nedges[i];
  }
  // largest instances first: the queue hands them out before the small ones
  std::vector<int> order(ninst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return inst[a].n > inst[b].n; });
  std::vector<QaoaInst> sorted(ninst);
  qvmg_qaoa_batch b = new qvmg_qaoa_s();
  b->ninst = ninst;
  b->p = p;
  b->n.assign(nqubits, nqubits + ninst);
  b->state_off.assign(ninst, 0);
  for (int r = 0; r < ninst; ++r) {
    QaoaInst q = inst[order[r]];
    q.state_off = soff;
    q.sub_off = uoff;
    q.cut_off = coff;  // multiples of 2^14: 16-byte aligned
    if (q.n > kQaoaTileBits) coff += 1ull << q.n;
    b->state_off[q.id] = soff;
    soff += 1ull << q.n;
    int sb = q.n < kQaoaSubBits ? q.n : kQaoaSubBits;
    uoff += 1ull << (q.n - sb);
    sorted[r] = q;
  }
  size_t ib = sizeof(QaoaInst) * ninst, eb = (e8.size() + 15) & ~(size_t)15,
         pb = sizeof(double) * (size_t)ninst * p;
  std::vector<unsigned char> host(ib + eb + 2 * pb, 0);
  std::memcpy(host.data(), sorted.data(), ib);
  if (!e8.empty()) std::memcpy(host.data() + ib, e8.data(), e8.size());
  std::memcpy(host.data() + ib + eb, gammas, pb);
  std::memcpy(host.data() + ib + eb + pb, betas, pb);
  cudaError_t e;
#define QCHK(call, what)                         \
  if ((e = (call)) != cudaSuccess) {             \
    int rc = cuda_fail(e, what);                 \
    qaoa_release(b);                             \
    return rc;                                   \
  }
  QCHK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  QCHK(cudaMalloc(&b->dbuf, host.size()), "cudaMalloc(batch tables)");
  // On the batch's own stream, then wait: a plain cudaMemcpy from pageable
  // memory can return before its DMA lands, on a stream the batch's
  // non-blocking stream does not wait for.
  QCHK(cudaMemcpyAsync(b->dbuf, host.data(), host.size(), cudaMemcpyHostToDevice, b->stream),
       "cudaMemcpyAsync(batch tables)");
  QCHK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
  QCHK(cudaMalloc(&b->states, soff * sizeof(float2)), "cudaMalloc(batch states)");
  QCHK(cudaMalloc(&b->subs, uoff * sizeof(double)), "cudaMalloc(batch CDF)");
  QCHK(cudaMalloc(&b->cuts, coff ? coff : 16), "cudaMalloc(batch cut values)");
  QCHK(cudaMalloc(&b->expect, ninst * sizeof(double)), "cudaMalloc(expectations)");
  QCHK(cudaMalloc(&b->counter, sizeof(unsigned int)), "cudaMalloc(counter)");
#undef QCHK
  b->bytes = host.size() + soff * sizeof(float2) + uoff * sizeof(double) + coff + ninst * 8;
  QaoaArgs &A = b->args;
  A.ninst = ninst;
  A.p = p;
  A.inst = (const QaoaInst *)b->dbuf;
  A.edges = (const unsigned char *)b->dbuf + ib;
  A.gammas = (const double *)((unsigned char *)b->dbuf + ib + eb);
  A.betas = (const double *)((unsigned char *)b->dbuf + ib + eb + pb);
  A.states = b->states;
  A.subs = b->subs;
  A.cuts = b->cuts;
  A.expect = b->expect;
  A.counter = b->counter;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  e = once(attr_once, attr_err, [] {
    const int bytes = (1 << kQaoaTileBits) * 8 + (kQaoaMaxEdges + 1) * 8 + 2 * kQaoaMaxEdges +
                      (1 << kQaoaTileBits) + 16;
    return cudaFuncSetAttribute(k_qaoa_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  if (e != cudaSuccess) {
    qaoa_release(b);
    return cuda_fail(e, "cudaFuncSetAttribute(k_qaoa_batch)");
  }
  *out = b;
  return QVMG_OK;
}

int qvmg_qaoa_batch_set_angles(qvmg_qaoa_batch b, const double *gammas, const double *betas) {
  if (!b || !gammas || !betas) return fail(QVMG_E_INVALID, "null batch or angles");
  size_t pb = sizeof(double) * (size_t)b->ninst * b->p;
  QVMG_CUDA(cudaMemcpyAsync((void *)b->args.gammas, gammas, pb, cudaMemcpyHostToDevice, b->stream));
  QVMG_CUDA(cudaMemcpyAsync((void *)b->args.betas, betas, pb, cudaMemcpyHostToDevice, b->stream));
  QVMG_CUDA(cudaStreamSynchronize(b->stream));
  return QVMG_OK;
}

int qvmg_qaoa_batch_run(qvmg_qaoa_batch b, const double *draws, int nshots, double *expectations,
                        uint32_t *shots) {
  if (!b) return fail(QVMG_E_INVALID, "null batch");
  if (nshots < 0 || (nshots > 0 && (!draws || !shots)))
    return fail(QVMG_E_INVALID, "shots requested without draws or output");
  if (nshots > b->nshots_cap) {
    QVMG_CUDA(cudaStreamSynchronize(b->stream));
    // The cached graph holds the old buffers: drop it before they are freed,
    // and record the capacity only once both new buffers exist, so that a
    // failed allocation can never leave a graph that writes freed memory.
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    b->graph_shots = -1;
    cudaFree(b->draws);
    cudaFree(b->shots);
    b->draws = nullptr;
    b->shots = nullptr;
    b->nshots_cap = 0;
    void *d = nullptr, *sh = nullptr;
    cudaError_t e = alloc_fault_injected() ? cudaErrorMemoryAllocation
                                           : cudaMalloc(&d, sizeof(double) * (size_t)b->ninst * nshots);
    if (e == cudaSuccess)
      e = alloc_fault_injected()
              ? cudaErrorMemoryAllocation
              : cudaMalloc(&sh, sizeof(unsigned int) * (size_t)b->ninst * nshots);
    if (e != cudaSuccess) {
      cudaFree(d);
      cudaFree(sh);
      cudaGetLastError();
      return cuda_fail(e, "cudaMalloc(batch draws and shots)");
    }
    b->draws = (double *)d;
    b->shots = (unsigned int *)sh;
    b->nshots_cap = nshots;
  }
  QaoaArgs &A = b->args;
  A.nshots = nshots;
  A.draws = b->draws;
  A.shots = b->shots;
  if (nshots > 0)
    QVMG_CUDA(cudaMemcpyAsync(b->draws, draws, sizeof(double) * (size_t)b->ninst * nshots,
                              cudaMemcpyHostToDevice, b->stream));
  // The queue reset and the persistent kernel are one captured graph,
  // replayed on every run with the same shot count.
  if (!b->graph || b->graph_shots != nshots) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g;
    QVMG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->counter, 0, sizeof(unsigned int), b->stream);
    int smem = (1 << kQaoaTileBits) * 8 + (kQaoaMaxEdges + 1) * 8 + 2 * kQaoaMaxEdges +
               (1 << kQaoaTileBits) + 16;
    int grid = std::min(b->ninst, sm_count() * 3);
    k_qaoa_batch<<<grid, kQaoaThreads, smem, b->stream>>>(A);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) return cuda_fail(le, "k_qaoa_batch launch");
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
    b->graph_shots = nshots;
  }
  QVMG_CUDA(cudaGraphLaunch(b->graph, b->stream));
  if (expectations)
    QVMG_CUDA(cudaMemcpyAsync(expectations, b->expect, sizeof(double) * b->ninst,
                              cudaMemcpyDeviceToHost, b->stream));
  if (nshots > 0)
    QVMG_CUDA(cudaMemcpyAsync(shots, b->shots, sizeof(unsigned int) * (size_t)b->ninst * nshots,
                              cudaMemcpyDeviceToHost, b->stream));
  QVMG_CUDA(cudaStreamSynchronize(b->stream));
  return QVMG_OK;
}

int qvmg_qaoa_batch_state(qvmg_qaoa_batch b, int instance, double *amps) {
  if (!b || !amps) return fail(QVMG_E_INVALID, "null batch or buffer");
  if (instance < 0 || instance >= b->ninst) return fail(QVMG_E_INVALID, "instance out of range");
  uint64_t len = 1ull << b->n[instance];
  std::vector<float2> tmp(len);
  QVMG_CUDA(cudaMemcpyAsync(tmp.data(), b->states + b->state_off[instance], len * sizeof(float2),
                            cudaMemcpyDeviceToHost, b->stream));
  QVMG_CUDA(cudaStreamSynchronize(b->stream));
  for (uint64_t i = 0; i < len; ++i) {
    amps[2 * i] = tmp[i].x;
    amps[2 * i + 1] = tmp[i].y;
  }
  return QVMG_OK;
}

uint64_t qvmg_qaoa_batch_bytes(qvmg_qaoa_batch b) { return b ? b->bytes : 0; }

int qvmg_qaoa_batch_free(qvmg_qaoa_batch b) {
  qaoa_release(b);
  return QVMG_OK;
}

}  // extern "C"
