// tile.cu -- the fused shared-memory tile pass.
//
// One pass applies a sequence of fused gate blocks to the whole state with a
// single read and a single write of every amplitude.  The state is cut into
// 2^(n-t) tiles of 2^t amplitudes: tile bits 0..L-1 are global qubits 0..L-1
// (a 256-byte contiguous row), bits L..t-1 are the pass's chosen global
// qubits E[0..].  A CTA streams tiles into shared memory with 16-byte
// asynchronous copies (cp.async), applies every op of the pass there, and
// writes the tile back.  The ops run in stages:
//  - register stages: each of the 256 threads owns 2^R amplitudes of the
//    tile (R tile bits, the stage's "slots"; the other 8 bits index the
//    thread).  A run of 1- and 2-qubit dense blocks whose bits fit the slots
//    is applied entirely in registers -- fully unrolled complex FMAs with the
//    block matrix held in registers, no shared-memory traffic and no address
//    arithmetic per op;
//  - shared-memory stages: diagonal phase tables (read in place from global
//    memory; each index from tile bits and per-tile constant bits as the
//    planner laid out), permutations, and dense blocks, one group of 2^k
//    amplitudes per thread (two groups sharing 16-byte words for FP32 1-/2-
//    qubit blocks);
//  - tensor-core stages: merged 3- to 5-qubit blocks as tcgen05 MMAs in
//    bf16x3 (tile_tc).  When a pass ends with one, that op writes its
//    results straight into HBM and the tile buffer takes the CTA's next tile
//    while its MMAs run (the pass then has no store loop).
// In kernels with register stages shared memory is XOR-swizzled (bits 1..3
// of a tile index are XORed with bits 4..12 folded) so that the lanes of a
// warp spread over the banks in both the row-contiguous copies and the
// register-stage gathers.
// This is the GB300 form of the reference's per-gate complement iteration
// (src/wavefunction.lisp:155-306, src/compile-gate.lisp:23-209): the same
// gather -> matvec -> scatter, for many gates per HBM round trip.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <cstring>
#include <vector>

#include "cplx.h"
#include "internal.h"
#include "tile.h"

namespace qvmg {

// Bank swizzle: linear in the index bits (XOR), keeps bit 0 (16-byte pairs).
__host__ __device__ __forceinline__ unsigned swz(unsigned j) {
  return j ^ ((((j >> 4) ^ (j >> 7) ^ (j >> 10)) & 7u) << 1);
}

// Tile index -> shared-memory index: swizzled only in kernels with register
// stages (their gathers need it); the shared-memory ops alone do not.
template <bool S>
__device__ __forceinline__ unsigned sw(unsigned j) {
  return S ? swz(j) : j;
}

__device__ __forceinline__ unsigned inject0u(unsigned x, int q) {
  unsigned lo = x & ((1u << q) - 1u);
  return ((x >> q) << (q + 1)) | lo;
}

// ---- shared-memory ops -----------------------------------------------------------

// The threads that work on one tile (a tile CTA): the ops take their thread
// index, count and barrier from here rather than from the launch shape.
struct Team {
  unsigned id;        // thread index within the team
  unsigned n;         // threads in the team
  unsigned warp_sub;  // this warp's quarter of TMEM lanes (CTA warp index % 4)
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};

// FP32 1-/2-qubit block with 16-byte shared-memory accesses.  Tile bit 0
// pairs two amplitudes in one 16-byte word: if it is a target, a group's
// amplitudes c and c | b0 come in one load; otherwise each thread takes the
// two groups that differ in bit 0 and loads both with every access.  Half
// the load, store and address instructions of one 8-byte access per
// amplitude, with every output summed in the same order (bit-identical):
// 296 against 303 ms for the 30-qubit depth-20 circuit, 638 against 699 ms
// unfused.
// Where a pass's last op may write its output: straight into the state in
// HBM (element p of the tile at rowoff[p >> L] + (p & (2^L - 1))) instead of
// the tile, so that the pass needs no store loop.
struct TileOut {
  float2 *a;
  const unsigned long long *rowoff;
  int L;
  __device__ __forceinline__ float4 *at(unsigned p) const {
    return reinterpret_cast<float4 *>(a + rowoff[p >> L] + (p & ((1u << L) - 1u)));
  }
};

template <int K, int J0>
__device__ __forceinline__ void tile_dense_v4(float2 *tile, int t, const float2 *m,
                                              const unsigned *off, const int *sp, const Team &tm,
                                              const TileOut *out) {
  constexpr int D = 1 << K;
  float4 *t4 = reinterpret_cast<float4 *>(tile);
  if constexpr (J0 >= 0) {
    // the target on tile bit 0 is matrix bit J0: amplitudes c and c | (1 << J0)
    // share a 16-byte word.  sp[0] == 0; inject the other targets.
    const unsigned ngroups = 1u << (t - K);
    for (unsigned g = tm.id; g < ngroups; g += tm.n) {
      unsigned b = g << 1;
#pragma unroll
      for (int s = 1; s < K; ++s) b = inject0u(b, sp[s]);
      float2 v[D];
#pragma unroll
      for (int c = 0; c < D; ++c)
        if (!((c >> J0) & 1)) {
          const float4 w = t4[(b | off[c]) >> 1];
          v[c] = make_float2(w.x, w.y);
          v[c | (1 << J0)] = make_float2(w.z, w.w);
        }
      float2 o[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) cmac(acc, m[r * D + c], v[c]);
        o[r] = acc;
      }
#pragma unroll
      for (int r = 0; r < D; ++r)
        if (!((r >> J0) & 1)) {
          const float2 a = o[r], e = o[r | (1 << J0)];
          const float4 w = make_float4(a.x, a.y, e.x, e.y);
          if (out) __stcs(out->at(b | off[r]), w);
          else t4[(b | off[r]) >> 1] = w;
        }
    }
  } else {
    // no target on bit 0: the groups at b and b | 1 share every 16-byte word
    const unsigned npairs = 1u << (t - K - 1);
    for (unsigned g = tm.id; g < npairs; g += tm.n) {
      unsigned b = g << 1;
#pragma unroll
      for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
      float2 va[D], vb[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const float4 w = t4[(b | off[c]) >> 1];
        va[c] = make_float2(w.x, w.y);
        vb[c] = make_float2(w.z, w.w);
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 a = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) {
          cmac(a, m[r * D + c], va[c]);
          cmac(e, m[r * D + c], vb[c]);
        }
        const float4 w = make_float4(a.x, a.y, e.x, e.y);
        if (out) __stcs(out->at(b | off[r]), w);
        else t4[(b | off[r]) >> 1] = w;
      }
    }
  }
}

template <typename T, int K, bool S>
__device__ __forceinline__ void tile_dense(typename CT<T>::C *tile, int t, const TileOpDev &op,
                                           const typename CT<T>::C *mat, const Team &tm,
                                           const TileOut *out = nullptr) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.pos[i];
#pragma unroll
  for (int i = 1; i < K; ++i)
#pragma unroll
    for (int j = i; j > 0; --j)
      if (sp[j - 1] > sp[j]) {
        int x = sp[j];
        sp[j] = sp[j - 1];
        sp[j - 1] = x;
      }
  unsigned off[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    unsigned o = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1u << op.pos[j];
    off[c] = o;
  }
  // Small matrices (FP32 1-/2-qubit, FP64 1-qubit) are held in registers
  // across the group loop: 16 shared-memory loads per group saved for an
  // FP32 2-qubit block.  Wider ones, and every matrix in the kernels with
  // register stages (whose register budget those stages take), are read from
  // shared memory with broadcast loads.
  constexpr bool kHoist = !S && D * D * sizeof(C) <= 128;
  C mreg[kHoist ? D * D : 1];
  if constexpr (kHoist) {
#pragma unroll
    for (int i = 0; i < D * D; ++i) mreg[i] = mat[i];
  }
  if constexpr (std::is_same<T, float>::value && !S && K <= 2) {
    if (op.pos[0] == 0) tile_dense_v4<K, 0>(tile, t, mreg, off, sp, tm, out);
    else if (K == 2 && op.pos[K - 1] == 0) tile_dense_v4<K, K - 1>(tile, t, mreg, off, sp, tm, out);
    else tile_dense_v4<K, -1>(tile, t, mreg, off, sp, tm, out);
    return;
  }
  const unsigned ngroups = 1u << (t - K);
  for (unsigned g = tm.id; g < ngroups; g += tm.n) {
    unsigned b = g;
#pragma unroll
    for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
    C v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = tile[sw<S>(b | off[c])];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      C acc = CT<T>::make(0, 0);
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if constexpr (kHoist) cmac(acc, mreg[r * D + c], v[c]);
        else cmac(acc, mat[r * D + c], v[c]);
      }
      tile[sw<S>(b | off[r])] = acc;
    }
  }
}

template <typename T, int K, bool S>
__device__ __forceinline__ void tile_perm(typename CT<T>::C *tile, int t, const TileOpDev &op,
                                          const Team &tm) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.pos[i];
#pragma unroll
  for (int i = 1; i < K; ++i)
#pragma unroll
    for (int j = i; j > 0; --j)
      if (sp[j - 1] > sp[j]) {
        int x = sp[j];
        sp[j] = sp[j - 1];
        sp[j - 1] = x;
      }
  unsigned off[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    unsigned o = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1u << op.pos[j];
    off[c] = o;
  }
  const int nm = op.nmoved;
  const unsigned ngroups = 1u << (t - K);
  for (unsigned g = tm.id; g < ngroups; g += tm.n) {
    unsigned b = g;
#pragma unroll
    for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
    C v[D];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < nm) v[j] = tile[sw<S>(b | off[op.src[j]])];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < nm) tile[sw<S>(b | off[op.dst[j]])] = v[j];
  }
}

// Table index of tile element j: the out-of-tile bits (cidx, fixed per
// tile) plus the in-tile bits read as runs or bit by bit (TileDiagInfo).
__device__ __forceinline__ int diag_tile_index(const TileDiagInfo &di, const TileOpDev &op,
                                               int cidx, unsigned j) {
  int idx = cidx;
  if (di.nruns != 255) {
    for (int r = 0; r < di.nruns; ++r)
      idx |= (int)((j >> di.run_t[r]) & ((1u << di.run_n[r]) - 1u)) << di.run_i[r];
  } else {
    for (int i = 0; i < op.k; ++i)
      if (di.tpos[i] != 255) idx |= (int)((j >> di.tpos[i]) & 1u) << i;
  }
  return idx;
}

// The out-of-tile index bits of this tile (from its base address, the
// offset of row 0), or -1 if a required qubit outside the tile is 0 here
// (every entry the tile would use is 1).
__device__ __forceinline__ int diag_tile_const(const TileDiagInfo &di, const TileOpDev &op,
                                               const unsigned long long *rowoff) {
  const unsigned long long base = rowoff[0];
  int cidx = 0;
  for (int i = 0; i < op.k; ++i)
    if (di.tpos[i] == 255) cidx |= (int)((base >> op.pos[i]) & 1ull) << i;
  return (cidx & di.out_req) == di.out_req ? cidx : -1;
}

// u-th element with the required in-tile bits set (ascending positions).
__device__ __forceinline__ unsigned diag_tile_element(const TileDiagInfo &di, unsigned u) {
  for (int r = 0; r < di.nreq; ++r) {
    const unsigned q = di.req_t[r];
    u = ((u >> q) << (q + 1)) | (1u << q) | (u & ((1u << q) - 1u));
  }
  return u;
}

// Whether a thread's table index is the same for all its elements.  Thread
// x takes elements u = x + k * nthreads (count and nthreads powers of two);
// inserting the required bits is linear over disjoint bits, so its elements
// differ only in the tile bits that the u bits at and above log2(nthreads)
// land on.  If the table holds none of those bits, one lookup serves them all.
__device__ __forceinline__ bool diag_thread_constant(const TileDiagInfo &di, const TileOpDev &op,
                                                     unsigned count, unsigned nthreads) {
  const unsigned uvary = (count - 1u) & ~(nthreads - 1u);
  const unsigned vmask = diag_tile_element(di, uvary) & ~diag_tile_element(di, 0u);
  unsigned tmask = 0;
  for (int i = 0; i < op.k; ++i)
    if (di.tpos[i] != 255) tmask |= 1u << di.tpos[i];
  return (tmask & vmask) == 0;
}

// The threads of a team that take part in a diagonal op: the largest power
// of two not above the team's size (the thread-constant test above needs a
// power-of-two stride; tensor-core CTAs have 288 threads).
__device__ __forceinline__ unsigned diag_threads(const Team &tm) {
  return 1u << (31 - __clz(tm.n));
}

// Diagonal op: each element's table entry multiplies it (entries of 1 are
// skipped).  The table is read in place from global memory through the
// read-only cache: staging a pass's tables in shared memory (a QFT chain
// takes up to 3 x 1024 entries) left room for one CTA per SM.  Where a
// thread's entry is the same for all its elements (two of the three tables
// of a QFT chain), it is read once.
template <typename T, bool S>
__device__ __forceinline__ void tile_diag(typename CT<T>::C *tile, int t, int L,
                                          const unsigned long long *rowoff, const TileOpDev &op,
                                          const typename CT<T>::C *table, const Team &tm) {
  using C = typename CT<T>::C;
  const TileDiagInfo &di = *reinterpret_cast<const TileDiagInfo *>(op.src);
  const int cidx = diag_tile_const(di, op, rowoff);
  if (cidx < 0) return;
  const unsigned count = (1u << t) >> di.nreq;
  const unsigned nt = diag_threads(tm);
  if (tm.id >= count || tm.id >= nt) return;
  if (diag_thread_constant(di, op, count, nt)) {
    const C ph = __ldg(table + diag_tile_index(di, op, cidx, diag_tile_element(di, tm.id)));
    if (ph.x == (T)1 && ph.y == (T)0) return;
    for (unsigned u = tm.id; u < count; u += nt) {
      const unsigned p = sw<S>(diag_tile_element(di, u));
      tile[p] = cmul(tile[p], ph);
    }
    return;
  }
  for (unsigned u = tm.id; u < count; u += nt) {
    const unsigned j = diag_tile_element(di, u);
    const C ph = __ldg(table + diag_tile_index(di, op, cidx, j));
    if (ph.x != (T)1 || ph.y != (T)0) {
      const unsigned p = sw<S>(j);
      tile[p] = cmul(tile[p], ph);
    }
  }
}

// ---- register stages (FP32) ---------------------------------------------------------

// 1-qubit block on register slot S of 2^R registers.
template <int R, int S>
__device__ __forceinline__ void reg_op1(float2 *v, const float2 *m) {
  const float2 m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
#pragma unroll
  for (int g = 0; g < (1 << (R - 1)); ++g) {
    const int b = ((g >> S) << (S + 1)) | (g & ((1 << S) - 1));
    const float2 a0 = v[b], a1 = v[b | (1 << S)];
    float2 r0 = cmul(m00, a0), r1 = cmul(m10, a0);
    cmac(r0, m01, a1);
    cmac(r1, m11, a1);
    v[b] = r0;
    v[b | (1 << S)] = r1;
  }
}

// 2-qubit block on register slots S0 < S1 (matrix index bit 0 <-> S0).
template <int R, int S0, int S1>
__device__ __forceinline__ void reg_op2(float2 *v, const float2 *m) {
  float2 mm[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) mm[i] = m[i];
#pragma unroll
  for (int g = 0; g < (1 << (R - 2)); ++g) {
    int b = ((g >> S0) << (S0 + 1)) | (g & ((1 << S0) - 1));
    b = ((b >> S1) << (S1 + 1)) | (b & ((1 << S1) - 1));
    const int i1 = b | (1 << S0), i2 = b | (1 << S1), i3 = b | (1 << S0) | (1 << S1);
    const float2 a0 = v[b], a1 = v[i1], a2 = v[i2], a3 = v[i3];
    float2 r[4];
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      float2 acc = cmul(mm[row * 4], a0);
      cmac(acc, mm[row * 4 + 1], a1);
      cmac(acc, mm[row * 4 + 2], a2);
      cmac(acc, mm[row * 4 + 3], a3);
      r[row] = acc;
    }
    v[b] = r[0];
    v[i1] = r[1];
    v[i2] = r[2];
    v[i3] = r[3];
  }
}

template <int R>
__device__ __forceinline__ void reg_apply(float2 *v, const TileOpDev &op, const float2 *m) {
  if (op.k == 1) {
    switch (op.slot0) {
      case 0: reg_op1<R, 0>(v, m); break;
      case 1: reg_op1<R, 1>(v, m); break;
      case 2: reg_op1<R, 2>(v, m); break;
      case 3: reg_op1<R, 3>(v, m); break;
      case 4: if constexpr (R > 4) reg_op1<R, 4>(v, m); break;
    }
    return;
  }
  switch (op.slot0 * 8 + op.slot1) {
    case 0 * 8 + 1: reg_op2<R, 0, 1>(v, m); break;
    case 0 * 8 + 2: reg_op2<R, 0, 2>(v, m); break;
    case 0 * 8 + 3: reg_op2<R, 0, 3>(v, m); break;
    case 1 * 8 + 2: reg_op2<R, 1, 2>(v, m); break;
    case 1 * 8 + 3: reg_op2<R, 1, 3>(v, m); break;
    case 2 * 8 + 3: reg_op2<R, 2, 3>(v, m); break;
    case 0 * 8 + 4: if constexpr (R > 4) reg_op2<R, 0, 4>(v, m); break;
    case 1 * 8 + 4: if constexpr (R > 4) reg_op2<R, 1, 4>(v, m); break;
    case 2 * 8 + 4: if constexpr (R > 4) reg_op2<R, 2, 4>(v, m); break;
    case 3 * 8 + 4: if constexpr (R > 4) reg_op2<R, 3, 4>(v, m); break;
  }
}

// A register stage: gather this thread's 2^R amplitudes, run the ops, scatter.
// The swizzle is linear, so swz(x | r) = swz(x) ^ swz(r) for disjoint bits.
template <int R>
__device__ __forceinline__ void reg_stage(float2 *tile, int t, const TileStageDev &st,
                                          const TileOpDev *ops, const float2 *data) {
  unsigned xb = 0;
  for (int i = 0; i < t - R; ++i)
    if ((threadIdx.x >> i) & 1u) xb |= 1u << st.tpos[i];
  const unsigned px = swz(xb);
  unsigned lo[4], hi[1 << (R - 2)];
#pragma unroll
  for (int r = 0; r < 4; ++r)
    lo[r] = swz(((r & 1) ? 1u << st.slots[0] : 0u) | ((r & 2) ? 1u << st.slots[1] : 0u)) ^ px;
#pragma unroll
  for (int h = 0; h < (1 << (R - 2)); ++h) {
    unsigned o = 0;
#pragma unroll
    for (int i = 0; i < R - 2; ++i)
      if ((h >> i) & 1) o |= 1u << st.slots[2 + i];
    hi[h] = swz(o);
  }
  float2 v[1 << R];
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) v[r] = tile[lo[r & 3] ^ hi[r >> 2]];
  for (int o = st.first; o < st.first + st.count; ++o) reg_apply<R>(v, ops[o], data + ops[o].data);
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) tile[lo[r & 3] ^ hi[r >> 2]] = v[r];
}

// ---- tensor-core ops (FP32 state, tcgen05, BF16x3) ----------------------------------
//
// A dense block on k = 3, 4 or 5 tile bits is a real GEMM per chunk of 128
// groups: D[g][n] = sum_kk A[g][kk] Bt[n][kk], with A[g] the group's 2^k
// amplitudes as (re, im) pairs and Bt the block's real form (n = 2r + re/im
// of output r).  Both operands are split into bf16 hi + lo parts and the
// three products that carry 16 significant bits are accumulated in FP32 in
// one tensor-memory accumulator:
//     D = Ahi*Bhi + Alo*Bhi + Ahi*Blo
// (the bf16x3 scheme; the dropped Alo*Blo term and the parts' own rounding
// are ~2^-17 relative).  A lives in tensor memory, written by the threads
// with tcgen05.st: TMEM lane g = group g, bf16 pairs packed two to a 32-bit
// column, the hi part in columns [0, D) and the lo part in [D, 2D).  Bt
// (split on the host) sits in the pass data in shared memory, K-major in
// 8-row x 16-byte core matrices, hi then lo.  Eight data warps serve a
// chunk, two threads per group: warps w and w+4 take the two halves of a
// group's amplitudes and write and read the matching columns of TMEM
// sub-partition w%4.  A ninth warp issues the MMAs, 3 per 16-element K step,
// and commits them to an mbarrier that the data warps wait on with a
// bounded loop.
//
// Chunks go in batches (two for 5-qubit blocks, four for 4-qubit ones, eight
// for 3-qubit ones), each chunk with its own TMEM buffer (D | A): a batch is
// gathered, its MMAs issued together under one commit, and read out after
// one wait -- two barriers per batch.
constexpr int kTcCols = 256;  // TMEM columns per CTA
// Test hook (qvmg_debug_tc_withhold): the MMA-issuing warp issues nothing,
// so the data warps' bounded wait runs out.
__device__ int g_tc_withhold = 0;
// A chunk of a k-qubit block takes 4 * 2^k TMEM columns: D (2^(k+1) FP32
// outputs) then A (2^k columns of hi, 2^k of lo, bf16 pairs); a batch is as
// many chunks as the CTA's columns hold (2 for k = 5, 4 for k = 4, 8 for
// k = 3: on a 13-qubit tile, a whole op).
constexpr int kTcWaitLimit = 1 << 20;  // tries of an MMA barrier wait before giving up

struct TcCtx {
  uint32_t tmem;      // TMEM address of lane 0, column 0 of this CTA's allocation
  uint32_t mbar[2];   // shared addresses of the two MMA-completion barriers
  uint32_t phase[2];  // parity of the phase each barrier's next wait is for
  int ok;             // 0 once a wait gave up
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: K-major, no swizzle; the next 16-byte
// core matrix along K is 128 bytes on, the next 8 rows `sbo` bytes on.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D[tmem] (+)= A[tmem] * B[smem]^T, bf16 operands, FP32 accumulation.
__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
      "r"(a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

template <int NR>
__device__ __forceinline__ void tmem_st(uint32_t taddr, const uint32_t (&r)[NR]);
template <>
__device__ __forceinline__ void tmem_st<4>(uint32_t taddr, const uint32_t (&r)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};\n" ::"r"(taddr),
               "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3])
               : "memory");
}
template <>
__device__ __forceinline__ void tmem_st<8>(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"r"(
                   taddr),
               "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),
               "r"(r[7])
               : "memory");
}

template <>
__device__ __forceinline__ void tmem_st<16>(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

template <int NR>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[NR]);
template <>
__device__ __forceinline__ void tmem_ld<32>(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Bounded wait for the barrier phase of parity `phase`; 1 when it completed.
// Each try may suspend the thread for up to 1 us until the phase completes
// (instead of spinning on issue slots the other CTA of the SM could use), so
// the whole wait gives up after at most ~1 s.
__device__ __forceinline__ uint32_t tc_wait(uint32_t mbar, uint32_t phase) {
  uint32_t done = 0;
  for (int it = 0; it < kTcWaitLimit && !done; ++it)
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase), "r"(1000u)
        : "memory");
  return done;
}

// bf16 hi/lo split of an amplitude (re, im): hi = bf16(x) (round to nearest
// even), lo = bf16(x - hi); each pair packed with re in the low half.
__device__ __forceinline__ void bf16_split(float2 v, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(v.x - hf.x, v.y - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

// Where the last op of a tensor-core pass puts its results: straight into
// the state in HBM instead of back into the tile (the pass then skips its
// store loop), and, once every chunk has been gathered, the tile buffer
// takes the next tile's loads while the MMAs and the readout run.
struct TcOut {
  float2 *a;                      // the state
  unsigned long long base;        // global index of this tile's element 0
  const unsigned long long *dep;  // row r of a tile sits at base | dep[r]
  int L;                          // row bits (2^L contiguous amplitudes)
  bool next;                      // a next tile to load
  unsigned long long next_base;
};

// The loads of a tile into the tile buffer: 16-byte asynchronous copies of
// its rows, every copy of the team in flight at once.
__device__ __forceinline__ void tile_load_async(float2 *tile, int t, const float2 *a,
                                                unsigned long long base,
                                                const unsigned long long *dep, int L,
                                                const Team &tm) {
  const unsigned nchunks = (1u << t) / 2, rowmask = (1u << L) - 1u;
  for (unsigned ch = tm.id; ch < nchunks; ch += tm.n) {
    const unsigned el = 2 * ch;
    cp_async16(tile + el, a + (base | dep[el >> L]) + (el & rowmask));
  }
}

template <int K>
__device__ __forceinline__ void tile_tc(float2 *tile, int t, const TileOpDev &op,
                                        const unsigned char *bmat, TcCtx &ctx,
                                        volatile int *abort_flag, const Team &tm,
                                        const TcOut *out) {
  constexpr int D = 1 << K, NC = 2 * D, H = D / 2;
  constexpr uint32_t kSboB = 2 * 16 * D;   // Bt rows hold 2D bf16 (4D bytes); 8 rows per group
  constexpr uint32_t kPieceB = 8 * D * D;  // bytes of Bt hi (then Bt lo)
  constexpr int kSteps = NC / 16;          // 16-element K steps per piece (8 TMEM columns)
  constexpr int kBufCols = 4 * D, kACol = 2 * D;  // per chunk: D | A hi | A lo
  constexpr unsigned kBufs = kTcCols / kBufCols;  // chunks per batch
  const int warp = (int)(tm.id >> 5), lane = (int)(tm.id & 31);
  const bool issuer = warp == kTileThreads / 32;  // the extra warp issues the MMAs
  // a warp reaches the TMEM lanes of its quarter: CTA warp index mod 4
  const int sub = (int)tm.warp_sub, half = (warp >> 2) & 1;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.pos[i];
#pragma unroll
  for (int i = 1; i < K; ++i)
#pragma unroll
    for (int j = i; j > 0; --j)
      if (sp[j - 1] > sp[j]) {
        const int x = sp[j];
        sp[j] = sp[j - 1];
        sp[j - 1] = x;
      }
  unsigned off[H];  // this thread's half of the group: amplitudes half*H .. half*H + H-1
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const int c = half * H + i;
    unsigned o = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if ((c >> j) & 1) o |= 1u << op.pos[j];
    off[i] = o;
  }
  // instruction descriptor: D f32, A and B bf16, both K-major, N = NC, M = 128
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NC >> 3) << 17) |
                         ((uint32_t)(kTileTcRows >> 4) << 24);
  const uint32_t lanes = (uint32_t)(sub * 32) << 16;
  const uint32_t bhi = smem_u32(bmat);
  const unsigned nchunks = (1u << (t - K)) / kTileTcRows;
  // Inserting the block's zero bits is linear over disjoint bit sets, so a
  // group's base is this thread's row part OR the chunk part (computed once).
  auto inject_all = [&](unsigned x) {
#pragma unroll
    for (int s = 0; s < K; ++s) x = inject0u(x, sp[s]);
    return x;
  };
  const unsigned row_base = inject_all((unsigned)(sub * 32 + lane));
  auto group_base = [&](unsigned ch) { return row_base | inject_all(ch * kTileTcRows); };
  // Chunks go in batches of up to kBufs: the data warps gather and split a
  // whole batch into its TMEM buffers, one barrier hands it to the issuing
  // warp, which issues every chunk's MMAs (each chunk on its own
  // accumulator) under one commit, and the data warps read out and scatter
  // the batch after one wait.  Two barriers per batch, the MMAs of all its
  // chunks in flight together.
  for (unsigned base = 0; base < nchunks; base += kBufs) {
    const unsigned nb = nchunks - base < kBufs ? nchunks - base : kBufs;
    if (!issuer) {
      for (unsigned c = 0; c < nb; ++c) {
        const uint32_t buf = ctx.tmem + c * kBufCols;
        const unsigned b = group_base(base + c);
        uint32_t hi[H], lo[H];
#pragma unroll
        for (int i = 0; i < H; ++i) bf16_split(tile[b | off[i]], hi[i], lo[i]);
        tmem_st<H>(buf + lanes + kACol + half * H, hi);
        tmem_st<H>(buf + lanes + kACol + D + half * H, lo);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    tm.sync();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (*abort_flag) {  // uniform: read after the barrier
      ctx.ok = 0;
      ctx.phase[0] ^= 1u;  // back to the phase of the commit that was not seen
      return;
    }
    // every chunk gathered: a last op hands the tile buffer to the next tile
    const bool load_next = out && out->next && base + kBufs >= nchunks;
    if (load_next && !issuer)
      tile_load_async(tile, t, out->a, out->next_base, out->dep, out->L, tm);
    if (issuer) {
      if (lane == 0 && !g_tc_withhold) {
        for (unsigned c = 0; c < nb; ++c) {
          const uint32_t buf = ctx.tmem + c * kBufCols;
          const uint32_t a = buf + kACol;
#pragma unroll
          for (int s = 0; s < kSteps; ++s)  // Ahi * Bhi
            tc_mma(buf, a + 8 * s, tc_desc(bhi + s * 256, kSboB), idesc, s > 0);
#pragma unroll
          for (int s = 0; s < kSteps; ++s)  // + Alo * Bhi
            tc_mma(buf, a + D + 8 * s, tc_desc(bhi + s * 256, kSboB), idesc, 1);
#pragma unroll
          for (int s = 0; s < kSteps; ++s)  // + Ahi * Blo
            tc_mma(buf, a + 8 * s, tc_desc(bhi + kPieceB + s * 256, kSboB), idesc, 1);
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                ctx.mbar[0])
            : "memory");
      }
      if (load_next) tile_load_async(tile, t, out->a, out->next_base, out->dep, out->L, tm);
    } else {
      if (!tc_wait(ctx.mbar[0], ctx.phase[0])) {
        *abort_flag = 1;  // seen by every thread after the next barrier
      } else {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        for (unsigned c = 0; c < nb; ++c) {
          uint32_t r[D];
          tmem_ld<D>(ctx.tmem + c * kBufCols + lanes + half * D, r);
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          const unsigned b = group_base(base + c);
          if (out) {
            // into HBM: the row deposit is linear over the disjoint bits of
            // the group base and the block offset
            const unsigned rowmask = (1u << out->L) - 1u;
            float2 *g = out->a + (out->base | out->dep[b >> out->L]);
#pragma unroll
            for (int i = 0; i < H; ++i)
              g[out->dep[off[i] >> out->L] + ((b | off[i]) & rowmask)] =
                  make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
          } else {
#pragma unroll
            for (int i = 0; i < H; ++i)
              tile[b | off[i]] =
                  make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
          }
        }
      }
    }
    ctx.phase[0] ^= 1u;  // every thread: the barrier's next phase
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    tm.sync();  // the batch's buffers are read out before the next one is written
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  }
  if (*abort_flag) {  // a wait that gave up on the last batch (seen after its barrier)
    ctx.ok = 0;
    ctx.phase[0] ^= 1u;
  }
}

// ---- double-float ops (fused FP64 tiles) -----------------------------------------

// Element type of the state in HBM: the tile's own type, except for
// double-float tiles, whose state stays complex FP64.
template <typename T>
struct GT {
  using G = typename CT<T>::C;
};
template <>
struct GT<dfloat> {
  using G = double2;
};
template <typename T>
constexpr bool kIsDf = std::is_same<T, dfloat>::value;

template <int K, bool S>
__device__ __forceinline__ void tile_dense_df(dfc *tile, int t, const Team &tm, const TileOpDev &op,
                                              const dfc *mat) {
  constexpr int D = 1 << K;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.pos[i];
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
      if ((c >> j) & 1) o |= 1u << op.pos[j];
    off[c] = o;
  }
  constexpr bool kHoist = K == 1;  // 4 entries in registers; wider ones broadcast from smem
  dfc mreg[kHoist ? D * D : 1];
  if constexpr (kHoist) {
#pragma unroll
    for (int i = 0; i < D * D; ++i) mreg[i] = mat[i];
  }
  const unsigned ngroups = 1u << (t - K);
  for (unsigned g = tm.id; g < ngroups; g += tm.n) {
    unsigned b = g;
#pragma unroll
    for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
    dfc v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = tile[sw<S>(b | off[c])];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      dfacc acc{0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if constexpr (kHoist) df_cmac(acc, mreg[r * D + c], v[c]);
        else df_cmac(acc, mat[r * D + c], v[c]);
      }
      tile[sw<S>(b | off[r])] = df_result(acc);
    }
  }
}

template <bool S>
__device__ __forceinline__ void tile_diag_df(dfc *tile, int t, int L,
                                             const unsigned long long *rowoff, const TileOpDev &op,
                                             const dfc *table, const Team &tm) {
  const TileDiagInfo &di = *reinterpret_cast<const TileDiagInfo *>(op.src);
  const int cidx = diag_tile_const(di, op, rowoff);
  if (cidx < 0) return;
  const unsigned count = (1u << t) >> di.nreq;
  const unsigned nt = diag_threads(tm);
  if (tm.id >= count || tm.id >= nt) return;
  if (diag_thread_constant(di, op, count, nt)) {
    const float4 e = __ldg(reinterpret_cast<const float4 *>(table) +
                           diag_tile_index(di, op, cidx, diag_tile_element(di, tm.id)));
    if (e.x == 1.f && e.y == 0.f && e.z == 0.f && e.w == 0.f) return;
    const dfc ph{e.x, e.y, e.z, e.w};
    for (unsigned u = tm.id; u < count; u += nt) {
      const unsigned p = sw<S>(diag_tile_element(di, u));
      tile[p] = df_cmul(tile[p], ph);
    }
    return;
  }
  for (unsigned u = tm.id; u < count; u += nt) {
    const unsigned j = diag_tile_element(di, u);
    const float4 e =
        __ldg(reinterpret_cast<const float4 *>(table) + diag_tile_index(di, op, cidx, j));
    if (e.x == 1.f && e.y == 0.f && e.z == 0.f && e.w == 0.f) continue;
    const unsigned p = sw<S>(j);
    tile[p] = df_cmul(tile[p], dfc{e.x, e.y, e.z, e.w});
  }
}

template <typename T, int KMAX, bool S>
__device__ __forceinline__ void smem_op(typename CT<T>::C *tile, int t, int L,
                                        const unsigned long long *rowoff, const TileOpDev &op,
                                        const typename CT<T>::C *md, const void *tables,
                                        const Team &tm) {
  // diagonal tables are read from global memory (op.data: entry offset)
  const typename CT<T>::C *gt = reinterpret_cast<const typename CT<T>::C *>(tables) + op.data;
  if (op.kind == 2) {
    switch (op.k) {
      case 1: tile_perm<T, 1, S>(tile, t, op, tm); break;
      case 2: tile_perm<T, 2, S>(tile, t, op, tm); break;
      case 3: if constexpr (KMAX >= 3) tile_perm<T, 3, S>(tile, t, op, tm); break;
      case 4: if constexpr (KMAX >= 4) tile_perm<T, 4, S>(tile, t, op, tm); break;
      case 5: if constexpr (KMAX >= 5) tile_perm<T, 5, S>(tile, t, op, tm); break;
    }
    return;
  }
  if constexpr (kIsDf<T>) {
    if (op.kind == 0) {
      switch (op.k) {
        case 1: tile_dense_df<1, S>(tile, t, tm, op, md); break;
        case 2: tile_dense_df<2, S>(tile, t, tm, op, md); break;
        case 3: if constexpr (KMAX >= 3) tile_dense_df<3, S>(tile, t, tm, op, md); break;
        case 4: if constexpr (KMAX >= 4) tile_dense_df<4, S>(tile, t, tm, op, md); break;
        case 5: if constexpr (KMAX >= 5) tile_dense_df<5, S>(tile, t, tm, op, md); break;
      }
    } else {
      tile_diag_df<S>(tile, t, L, rowoff, op, gt, tm);
    }
  } else {
    if (op.kind == 0) {
      switch (op.k) {
        case 1: tile_dense<T, 1, S>(tile, t, op, md, tm); break;
        case 2: tile_dense<T, 2, S>(tile, t, op, md, tm); break;
        case 3: if constexpr (KMAX >= 3) tile_dense<T, 3, S>(tile, t, op, md, tm); break;
        case 4: if constexpr (KMAX >= 4) tile_dense<T, 4, S>(tile, t, op, md, tm); break;
        case 5: if constexpr (KMAX >= 5) tile_dense<T, 5, S>(tile, t, op, md, tm); break;
      }
    } else {
      tile_diag<T, S>(tile, t, L, rowoff, op, gt, tm);
    }
  }
}

// KMAX: widest op of the pass; RB: register bits of the register stages
// (0: every stage runs in shared memory; -1: the pass has tensor-core ops).
// Narrow instantiations keep the register arrays of wide cases out of the
// kernel.  Threads of a tile CTA: 128 for the FMA engine, 256 with register
// stages and for double-float tiles, 256 plus the MMA-issuing warp in
// tensor-core kernels.
template <typename T, int RB>
constexpr int tile_threads() {
  return RB == 0 && !kIsDf<T> ? kTileThreadsSmem : (RB < 0 ? kTileThreads + 32 : kTileThreads);
}

// A tile's global base index (its element 0) and the offset of its row r of
// 2^L contiguous amplitudes.
__device__ __forceinline__ unsigned long long tile_base_index(const TileArgs &p,
                                                              unsigned long long c) {
  unsigned long long base = c << p.L;
  for (int e = 0; e < p.nE; ++e) {
    const int q = p.E[e];
    const unsigned long long lo = base & ((1ull << q) - 1ull);
    base = ((base >> q) << (q + 1)) | lo;
  }
  return base;
}
__device__ __forceinline__ unsigned long long tile_row_offset(const TileArgs &p,
                                                              unsigned long long base, unsigned r) {
  unsigned long long o = base;
  for (int e = 0; e < p.nE; ++e)
    if ((r >> e) & 1u) o |= 1ull << p.E[e];
  return o;
}

template <typename T, int KMAX, int RB>
__global__ void __launch_bounds__(tile_threads<T, RB>(), (RB == 5 || RB < 0) ? 2 : (KMAX <= 2 ? 3 : 1))
    k_tile(typename GT<T>::G *__restrict__ a, const __grid_constant__ TileArgs p) {
  using C = typename CT<T>::C;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) unsigned long long tc_mbar[2];
  __shared__ uint32_t tc_tmem_slot;
  __shared__ int tc_abort;
  __shared__ unsigned long long tc_base;  // the tile's element 0 (a diagonal op's row offset 0)
  const Team tm{threadIdx.x, blockDim.x, (threadIdx.x >> 5) & 3u};
  TcCtx ctx{0u, {0u, 0u}, {0u, 0u}, 1};
  if constexpr (RB < 0) {
    if ((threadIdx.x >> 5) == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                       smem_u32(&tc_tmem_slot)),
                   "n"(kTcCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (threadIdx.x == 0) {
      tc_abort = 0;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&tc_mbar[0])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&tc_mbar[1])) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
  }
  const int t = p.t, L = p.L;
  C *tile = reinterpret_cast<C *>(smem);
  unsigned long long *rowoff = reinterpret_cast<unsigned long long *>(tile + (1u << t));
  const unsigned nrows = 1u << (t - L);
  // row offsets padded to 16 bytes so that double2 op data stays aligned
  C *data = reinterpret_cast<C *>(rowoff + ((nrows + 1u) & ~1u));
  TileOpDev *ops = reinterpret_cast<TileOpDev *>(data + p.ndata);
  TileStageDev *stages = reinterpret_cast<TileStageDev *>(ops + p.nops);
  {
    if constexpr (kIsDf<T>) {
      const double2 *gd = reinterpret_cast<const double2 *>(p.data);
      for (int i = threadIdx.x; i < p.ndata; i += blockDim.x) data[i] = df_from_double2_any(gd[i]);
    } else {
      const C *gd = reinterpret_cast<const C *>(p.data);
      for (int i = threadIdx.x; i < p.ndata; i += blockDim.x) data[i] = gd[i];
    }
    const int *gs = reinterpret_cast<const int *>(p.ops);
    int *ss = reinterpret_cast<int *>(ops);
    const int words = p.nops * (int)(sizeof(TileOpDev) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) ss[i] = gs[i];
    const int *gt = reinterpret_cast<const int *>(p.stages);
    int *st = reinterpret_cast<int *>(stages);
    const int swords = p.nstages * (int)(sizeof(TileStageDev) / 4);
    for (int i = threadIdx.x; i < swords; i += blockDim.x) st[i] = gt[i];
  }
  if constexpr (RB < 0) {
    // tensor-core passes keep the pass's row deposits (row r of a tile at
    // its base | rowoff[r]) instead of per-tile row offsets
    for (unsigned r = threadIdx.x; r < nrows; r += blockDim.x) rowoff[r] = tile_row_offset(p, 0ull, r);
    // the tensor core reads the operands in the pass data through the async proxy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    ctx.tmem = tc_tmem_slot;
    ctx.mbar[0] = smem_u32(&tc_mbar[0]);
    ctx.mbar[1] = smem_u32(&tc_mbar[1]);
  }
  constexpr int per16 = 16 / sizeof(C);  // amplitudes per 16-byte chunk
  const unsigned nchunks = (1u << t) / per16;
  const unsigned rowmask = (1u << L) - 1u;
  if constexpr (RB < 0) {
    // A pass whose last op is a tensor-core op writes its results from the
    // readout straight into HBM and loads the next tile under that op's
    // MMAs (TcOut); other passes store the tile afterwards.
    const float2 *ga = reinterpret_cast<const float2 *>(a);
    bool loaded = false;  // this tile's loads were issued by the previous tile's last op
    for (unsigned long long c = blockIdx.x; c < p.ntiles; c += gridDim.x) {
      // the previous tile's store loop is done with the buffer (a last op
      // that loaded this tile ended with its own barrier)
      if (!loaded) __syncthreads();
      const unsigned long long base = tile_base_index(p, c);
      if (threadIdx.x == 0) tc_base = base;
      if (!loaded) tile_load_async(reinterpret_cast<float2 *>(tile), t, ga, base, rowoff, L, tm);
      cp_async_wait_all();
      __syncthreads();
      const unsigned long long cn = c + gridDim.x;
      const bool has_next = cn < p.ntiles;
      bool direct = false;
      for (int s = 0; s < p.nstages; ++s) {
        const TileOpDev &op = ops[stages[s].first];
        if (op.kind == 3) {
          const unsigned char *bm = reinterpret_cast<const unsigned char *>(data + op.data);
          float2 *ft = reinterpret_cast<float2 *>(tile);
          const bool last = s == p.nstages - 1;
          const TcOut o{reinterpret_cast<float2 *>(a), base, rowoff, L, has_next,
                        has_next && last ? tile_base_index(p, cn) : 0ull};
          const TcOut *po = last ? &o : nullptr;
          if (op.k == 3) tile_tc<3>(ft, t, op, bm, ctx, &tc_abort, tm, po);
          else if (op.k == 4) tile_tc<4>(ft, t, op, bm, ctx, &tc_abort, tm, po);
          else tile_tc<5>(ft, t, op, bm, ctx, &tc_abort, tm, po);
          if (!ctx.ok) break;
          direct = last;  // tile_tc ends with a barrier after its readout
        } else {
          smem_op<T, KMAX, false>(tile, t, L, &tc_base, op, data + op.data, p.tables, tm);
          __syncthreads();
        }
      }
      if (!ctx.ok) break;  // uniform: set after a block-wide vote
      loaded = direct && has_next;
      if (!direct) {
        const unsigned rowmask = (1u << L) - 1u;
        for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
          const unsigned el = ch * per16;
          __stcs(reinterpret_cast<int4 *>(a + (base | rowoff[el >> L]) + (el & rowmask)),
                 *reinterpret_cast<const int4 *>(tile + el));
        }
      }
    }
    cp_async_wait_all();  // a tile loaded ahead lands before the CTA ends
  } else {
    // An FP32 FMA pass whose last op is a 1-/2-qubit dense block writes that
    // op's output pairs straight into HBM (TileOut): no store loop.
    bool direct = false;
    if constexpr (std::is_same<T, float>::value && RB == 0) {
      __syncthreads();  // the op and stage descriptors are in shared memory
      if (p.nstages > 0) {
        const TileOpDev &lop = ops[stages[p.nstages - 1].first];
        direct = lop.kind == 0 && lop.k <= 2;
      }
    }
    for (unsigned long long c = blockIdx.x; c < p.ntiles; c += gridDim.x) {
      __syncthreads();  // previous tile's stores done before rowoff/tile reuse
      const unsigned long long base = tile_base_index(p, c);
      for (unsigned r = threadIdx.x; r < nrows; r += blockDim.x)
        rowoff[r] = tile_row_offset(p, base, r);
      __syncthreads();
      for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
        unsigned el = ch * per16;
        const typename GT<T>::G *src = a + rowoff[el >> L] + (el & rowmask);
        cp_async16(tile + sw<(RB > 0)>(el), src);
      }
      cp_async_wait_all();
      if constexpr (kIsDf<T>) {
        // this thread's own copies have landed: FP64 -> double-float in place
        for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
          dfc &d = tile[ch];
          d = df_from_double2(*reinterpret_cast<const double2 *>(&d));
        }
      }
      __syncthreads();
      for (int s = 0; s < p.nstages; ++s) {
        const TileStageDev &st = stages[s];
        if constexpr (RB > 0) {
          if (st.reg) {
            reg_stage<RB>(reinterpret_cast<float2 *>(tile), t, st, ops,
                          reinterpret_cast<const float2 *>(data));
            __syncthreads();
            continue;
          }
        }
        const TileOpDev &op = ops[st.first];
        if constexpr (std::is_same<T, float>::value && RB == 0) {
          if (direct && s == p.nstages - 1) {
            const TileOut o{reinterpret_cast<float2 *>(a), rowoff, L};
            if (op.k == 1) tile_dense<float, 1, false>(tile, t, op, data + op.data, tm, &o);
            else tile_dense<float, 2, false>(tile, t, op, data + op.data, tm, &o);
            continue;  // the next tile's first barrier orders the buffer's reuse
          }
        }
        smem_op<T, KMAX, (RB > 0)>(tile, t, L, rowoff, op, data + op.data, p.tables, tm);
        __syncthreads();
      }
      if (direct) continue;
      for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
        unsigned el = ch * per16;
        int4 *dst = reinterpret_cast<int4 *>(a + rowoff[el >> L] + (el & rowmask));
        if constexpr (kIsDf<T>) {
          const double2 v = df_to_double2(tile[el]);
          __stcs(dst, *reinterpret_cast<const int4 *>(&v));
        } else {
          __stcs(dst, *reinterpret_cast<const int4 *>(tile + sw<(RB > 0)>(el)));
        }
      }
    }
  }
  if constexpr (RB < 0) {
    if (!ctx.ok) {
      if (threadIdx.x == 0) atomicExch(p.status, 1);
      // let MMAs still in flight finish (bounded) before their TMEM is freed
      (void)tc_wait(ctx.mbar[0], ctx.phase[0]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(ctx.tmem),
                   "n"(kTcCols)
                   : "memory");
  }
}

size_t tile_smem_bytes(int prec, int t, int L, int ndata, int nops, int nstages) {
  size_t csz = prec == QVMG_FP64 ? 16 : 8;
  size_t rows = ((size_t)1 << (t - L)) + 1 & ~(size_t)1;  // padded to 16 bytes
  size_t b = ((size_t)1 << t) * csz + rows * 8 + (size_t)ndata * csz +
             (size_t)nops * sizeof(TileOpDev) + (size_t)nstages * sizeof(TileStageDev);
  return (b + 15) & ~(size_t)15;
}

template <typename T, int KMAX, int RB>
static int tile_launch_k(qvmg_state s, const TileArgs &args, size_t smem) {
  static std::once_flag attr_once;  // per instantiation
  static cudaError_t attr_err = cudaSuccess;
  QVMG_CUDA(once(attr_once, attr_err, [] {
    cudaError_t e = cudaFuncSetAttribute(k_tile<T, KMAX, RB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kTileMaxSmem);
    // the whole unified L1/shared array as shared memory: the occupancy
    // query (and the launch) then fit as many tiles per SM as the bytes allow
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tile<T, KMAX, RB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    return e;
  }));
  // Persistent grid: as many CTAs as fit on every SM at once (registers and
  // shared memory), each looping over tiles.
  int per_sm = 0;
  QVMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<T, KMAX, RB>,
                                                          tile_threads<T, RB>(), smem));
  if (per_sm < 1) return fail(QVMG_E_UNSUPPORTED, "tile pass does not fit on an SM");
  if (RB < 0) {
    // The occupancy query answers 1 for kernels that allocate tensor memory;
    // count what bounds co-resident CTAs ourselves: shared memory (with the
    // 1 KiB the runtime reserves per CTA), registers, and the 512 TMEM
    // columns of an SM.  (The persistent loop is correct for any grid.)
    static int smem_sm = 0, regs = 0, stat = 0;
    static std::once_flag info_once;
    static cudaError_t info_err = cudaSuccess;
    QVMG_CUDA(once(info_once, info_err, [] {
      int dev = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
      cudaFuncAttributes fa;
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_tile<T, KMAX, RB>);
      if (e == cudaSuccess) {
        regs = fa.numRegs;
        stat = (int)fa.sharedSizeBytes;
      }
      return e;
    }));
    const int by_smem = smem_sm / (int)(smem + (size_t)stat + 1024);
    const int by_regs = 65536 / (((regs * 32 + 255) / 256) * 256 * (tile_threads<T, RB>() / 32));
    per_sm = std::max(1, std::min(std::min(by_smem, by_regs), 512 / kTcCols));
  }
  uint64_t grid = std::min<uint64_t>(args.ntiles, (uint64_t)sm_count() * per_sm);
  // a yielding state (priority -1): short CTAs of 16 tiles each, so that the
  // block scheduler can start other streams' CTAs between them
  if (s->priority < 0) grid = std::max<uint64_t>(grid, args.ntiles / 16);
  k_tile<T, KMAX, RB><<<(unsigned)grid, tile_threads<T, RB>(), smem, s->stream>>>(
      (typename GT<T>::G *)s->amps, args);
  QVMG_CHECK_LAUNCH("k_tile");
  return QVMG_OK;
}

template <typename T, int RB>
static int tile_launch_r(qvmg_state s, const TileArgs &args, size_t smem) {
  if (args.kmax <= 2) return tile_launch_k<T, 2, RB>(s, args, smem);
  if (args.kmax <= 3) return tile_launch_k<T, 3, RB>(s, args, smem);
  return tile_launch_k<T, 5, RB>(s, args, smem);
}

int launch_tile(qvmg_state s, const TileArgs &args) {
  size_t smem = tile_smem_bytes(s->prec, args.t, args.L, args.ndata, args.nops, args.nstages);
  if (smem > (size_t)kTileMaxSmem) return fail(QVMG_E_UNSUPPORTED, "tile pass exceeds shared memory");
  if (args.kmax < 1 || args.kmax > 5) return fail(QVMG_E_INVALID, "tile op width out of range");
  if (s->prec == QVMG_FP64) {
    if (args.R != 0) return fail(QVMG_E_INVALID, "register stages are FP32 only");
    return tile_launch_r<dfloat, 0>(s, args, smem);
  }
  if (args.tc) {
    if (args.R != 0) return fail(QVMG_E_INVALID, "tensor-core passes have no register stages");
    if (!args.status) return fail(QVMG_E_INVALID, "tensor-core pass without a status word");
    return tile_launch_r<float, -1>(s, args, smem);
  }
  if (args.R == 5) return tile_launch_r<float, 5>(s, args, smem);
  if (args.R == 4) return tile_launch_r<float, 4>(s, args, smem);
  if (args.R == 0) return tile_launch_r<float, 0>(s, args, smem);
  return fail(QVMG_E_INVALID, "unsupported register-stage width");
}

}  // namespace qvmg

extern "C" int qvmg_debug_tc_withhold(int on) {
  const int v = on ? 1 : 0;
  QVMG_CUDA(cudaMemcpyToSymbol(qvmg::g_tc_withhold, &v, sizeof(int)));
  return QVMG_OK;
}
