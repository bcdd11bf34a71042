// tile.cu -- the fused shared-memory tile pass.
//
// One pass applies a sequence of fused gate blocks to the whole state with a
// single read and a single write of every amplitude.  The state is cut into
// 2^(n-t) tiles of 2^t amplitudes: tile-local bits 0..L-1 are global qubits
// 0..L-1 (a 256-byte contiguous row), bits L..t-1 are the pass's chosen
// global qubits E[0..].  A CTA loads a tile row by row with 16-byte vector
// loads into shared memory, applies every op of the pass there (dense k<=5
// blocks gathered into registers, permutations as register moves, diagonal
// phase tables indexed by the global address), then writes the rows back.
// This is the GB300 form of the reference's per-gate complement iteration
// (src/wavefunction.lisp:155-306, src/compile-gate.lisp:23-209): the same
// gather -> matvec -> scatter, but over shared memory for many gates at once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cplx.h"
#include "internal.h"
#include "tile.h"

namespace qvmg {

// 16-byte asynchronous global -> shared copy (LDGSTS): every load of a tile
// is in flight at once without holding registers; wait_all completes them.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

__device__ __forceinline__ unsigned inject0u(unsigned x, int q) {
  unsigned lo = x & ((1u << q) - 1u);
  return ((x >> q) << (q + 1)) | lo;
}

template <typename T, int K>
__device__ __forceinline__ void tile_dense(typename CT<T>::C *tile, int t, const TileOpDev &op,
                                           const typename CT<T>::C *mat) {
  using C = typename CT<T>::C;
  constexpr int D = 1 << K;
  int sp[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sp[i] = op.pos[i];
  // insertion sort (K <= 5)
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
  const unsigned ngroups = 1u << (t - K);
  if (K <= 2) {
    C m[D * D];
#pragma unroll
    for (int i = 0; i < D * D; ++i) m[i] = mat[i];
    for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x) {
      unsigned b = g;
#pragma unroll
      for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
      C v[D];
#pragma unroll
      for (int c = 0; c < D; ++c) v[c] = tile[b + off[c]];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        C acc = CT<T>::make(0, 0);
#pragma unroll
        for (int c = 0; c < D; ++c) cmac(acc, m[r * D + c], v[c]);
        tile[b + off[r]] = acc;
      }
    }
  } else {
    for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x) {
      unsigned b = g;
#pragma unroll
      for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
      C v[D];
#pragma unroll
      for (int c = 0; c < D; ++c) v[c] = tile[b + off[c]];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        C acc = CT<T>::make(0, 0);
#pragma unroll
        for (int c = 0; c < D; ++c) cmac(acc, mat[r * D + c], v[c]);
        tile[b + off[r]] = acc;
      }
    }
  }
}

template <typename T, int K>
__device__ __forceinline__ void tile_perm(typename CT<T>::C *tile, int t, const TileOpDev &op) {
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
  for (unsigned g = threadIdx.x; g < ngroups; g += blockDim.x) {
    unsigned b = g;
#pragma unroll
    for (int s = 0; s < K; ++s) b = inject0u(b, sp[s]);
    C v[D];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < nm) v[j] = tile[b + off[op.src[j]]];
#pragma unroll
    for (int j = 0; j < D; ++j)
      if (j < nm) tile[b + off[op.dst[j]]] = v[j];
  }
}

template <typename T>
__device__ __forceinline__ void tile_diag(typename CT<T>::C *tile, int t, int L,
                                          const unsigned long long *rowoff, const TileOpDev &op,
                                          const typename CT<T>::C *table) {
  using C = typename CT<T>::C;
  const unsigned n = 1u << t;
  const unsigned rowmask = (1u << L) - 1u;
  const int k = op.k;
  for (unsigned j = threadIdx.x; j < n; j += blockDim.x) {
    unsigned long long g = rowoff[j >> L] | (j & rowmask);
    int idx = 0;
    for (int i = 0; i < k; ++i) idx |= (int)((g >> op.pos[i]) & 1ull) << i;
    C ph = table[idx];
    if (ph.x != (T)1 || ph.y != (T)0) tile[j] = cmul(tile[j], ph);
  }
}

// KMAX: widest op of the pass; narrower instantiations keep the register
// arrays of the wide cases out of the kernel (no spills for k <= 2).
template <typename T, int KMAX>
__global__ void __launch_bounds__(kTileThreads, KMAX <= 2 ? 3 : 1)
    k_tile(typename CT<T>::C *__restrict__ a, const __grid_constant__ TileArgs p) {
  using C = typename CT<T>::C;
  extern __shared__ __align__(16) unsigned char smem[];
  const int t = p.t, L = p.L;
  C *tile = reinterpret_cast<C *>(smem);
  unsigned long long *rowoff = reinterpret_cast<unsigned long long *>(tile + (1u << t));
  const unsigned nrows = 1u << (t - L);
  // row offsets padded to 16 bytes so that double2 op data stays aligned
  C *data = reinterpret_cast<C *>(rowoff + ((nrows + 1u) & ~1u));
  TileOpDev *ops = reinterpret_cast<TileOpDev *>(data + p.ndata);
  {
    const C *gd = reinterpret_cast<const C *>(p.data);
    for (int i = threadIdx.x; i < p.ndata; i += blockDim.x) data[i] = gd[i];
    const int *gs = reinterpret_cast<const int *>(p.ops);
    int *ss = reinterpret_cast<int *>(ops);
    const int words = p.nops * (int)(sizeof(TileOpDev) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) ss[i] = gs[i];
  }
  constexpr int per16 = 16 / sizeof(C);  // amplitudes per 16-byte chunk
  const unsigned nchunks = (1u << t) / per16;
  const unsigned rowmask = (1u << L) - 1u;
  for (unsigned long long c = blockIdx.x; c < p.ntiles; c += gridDim.x) {
    __syncthreads();  // previous tile's stores done before rowoff/tile reuse
    unsigned long long base = c << L;
    for (int e = 0; e < p.nE; ++e) {
      int q = p.E[e];
      unsigned long long lo = base & ((1ull << q) - 1ull);
      base = ((base >> q) << (q + 1)) | lo;
    }
    for (unsigned r = threadIdx.x; r < nrows; r += blockDim.x) {
      unsigned long long o = base;
      for (int e = 0; e < p.nE; ++e)
        if ((r >> e) & 1u) o |= 1ull << p.E[e];
      rowoff[r] = o;
    }
    __syncthreads();
    for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
      unsigned el = ch * per16;
      const int4 *src = reinterpret_cast<const int4 *>(a + rowoff[el >> L] + (el & rowmask));
      cp_async16(reinterpret_cast<int4 *>(tile) + ch, src);
    }
    cp_async_wait_all();
    __syncthreads();
    for (int o = 0; o < p.nops; ++o) {
      const TileOpDev &op = ops[o];
      const C *md = data + op.data;
      if (op.kind == 0) {
        switch (op.k) {
          case 1: tile_dense<T, 1>(tile, t, op, md); break;
          case 2: tile_dense<T, 2>(tile, t, op, md); break;
          case 3: if constexpr (KMAX >= 3) tile_dense<T, 3>(tile, t, op, md); break;
          case 4: if constexpr (KMAX >= 4) tile_dense<T, 4>(tile, t, op, md); break;
          case 5: if constexpr (KMAX >= 5) tile_dense<T, 5>(tile, t, op, md); break;
        }
      } else if (op.kind == 2) {
        switch (op.k) {
          case 1: tile_perm<T, 1>(tile, t, op); break;
          case 2: tile_perm<T, 2>(tile, t, op); break;
          case 3: if constexpr (KMAX >= 3) tile_perm<T, 3>(tile, t, op); break;
          case 4: if constexpr (KMAX >= 4) tile_perm<T, 4>(tile, t, op); break;
          case 5: if constexpr (KMAX >= 5) tile_perm<T, 5>(tile, t, op); break;
        }
      } else {
        tile_diag<T>(tile, t, L, rowoff, op, md);
      }
      __syncthreads();
    }
    for (unsigned ch = threadIdx.x; ch < nchunks; ch += blockDim.x) {
      unsigned el = ch * per16;
      int4 *dst = reinterpret_cast<int4 *>(a + rowoff[el >> L] + (el & rowmask));
      __stcs(dst, reinterpret_cast<const int4 *>(tile)[ch]);
    }
  }
}

size_t tile_smem_bytes(int prec, int t, int L, int ndata, int nops) {
  size_t csz = prec == QVMG_FP64 ? 16 : 8;
  size_t rows = ((size_t)1 << (t - L)) + 1 & ~(size_t)1;  // padded to 16 bytes
  size_t b = ((size_t)1 << t) * csz + rows * 8 + (size_t)ndata * csz +
             (size_t)nops * sizeof(TileOpDev);
  return (b + 15) & ~(size_t)15;
}

template <typename T, int KMAX>
static int tile_launch_k(qvmg_state s, const TileArgs &args, size_t smem) {
  static bool attr = false;  // per instantiation
  if (!attr) {
    QVMG_CUDA(cudaFuncSetAttribute(k_tile<T, KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kTileMaxSmem));
    attr = true;
  }
  // Persistent grid: as many CTAs as fit on every SM at once (registers and
  // shared memory), each looping over tiles.
  int per_sm = 0;
  QVMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<T, KMAX>, kTileThreads,
                                                          smem));
  if (per_sm < 1) return fail(QVMG_E_UNSUPPORTED, "tile pass does not fit on an SM");
  uint64_t grid = std::min<uint64_t>(args.ntiles, (uint64_t)sm_count() * per_sm);
  k_tile<T, KMAX><<<(unsigned)grid, kTileThreads, smem, s->stream>>>(
      (typename CT<T>::C *)s->amps, args);
  QVMG_CHECK_LAUNCH("k_tile");
  return QVMG_OK;
}

template <typename T>
static int tile_launch(qvmg_state s, const TileArgs &args, size_t smem) {
  if (args.kmax <= 2) return tile_launch_k<T, 2>(s, args, smem);
  if (args.kmax <= 3) return tile_launch_k<T, 3>(s, args, smem);
  return tile_launch_k<T, 5>(s, args, smem);
}

int launch_tile(qvmg_state s, const TileArgs &args) {
  size_t smem = tile_smem_bytes(s->prec, args.t, args.L, args.ndata, args.nops);
  if (smem > (size_t)kTileMaxSmem) return fail(QVMG_E_UNSUPPORTED, "tile pass exceeds shared memory");
  if (args.kmax < 1 || args.kmax > 5) return fail(QVMG_E_INVALID, "tile op width out of range");
  if (s->prec == QVMG_FP64) return tile_launch<double>(s, args, smem);
  return tile_launch<float>(s, args, smem);
}

}  // namespace qvmg
