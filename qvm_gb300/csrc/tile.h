// tile.h -- device descriptors of a shared-memory tile pass.
#pragma once
#include <stdint.h>

#include "internal.h"

namespace qvmg {

constexpr int kTileThreads = 256;  // register-stage and tensor-core kernels
// FP32 kernels whose ops all run over shared memory (the FMA engine).  Every
// thread repeats each op's setup (sorted positions, offsets, the hoisted
// block matrix) for every tile, so fewer threads per tile do less of it: 128
// threads and 3 CTAs per SM took the 30-qubit depth-20 circuit from 296 to
// 278 ms (256 and 192 threads, and 64 threads with 6-8 CTAs per SM, were
// slower at 13-qubit tiles).  FP64 double-float tiles keep 256 threads: 128
// took the fused 28-qubit circuit from 522 to 537 ms.
constexpr int kTileThreadsSmem = 128;
// Dynamic shared memory of a tile pass: the 227 KiB a CTA may hold, less
// 128 bytes for the kernel's static shared variables (MMA barriers, TMEM slot).
constexpr int kTileMaxSmem = 227 * 1024 - 128;
constexpr int kTileMaxE = 24;
constexpr int kTileTcRows = 128;  // groups per tensor-core chunk (MMA M)

// One op of a tile pass (128 bytes, copied into shared memory as words).
struct TileOpDev {
  int kind;  // 0 dense, 1 diagonal table, 2 permutation, 3 tensor-core dense
  int k;     // qubits
  int data;  // offset (complex elements) of the matrix / table in pass data
  int nmoved;
  int pos[10];  // dense/perm: tile-local bit positions; diag: global qubits (nat order)
  int slot0, slot1;  // register-stage ops: register slots of pos[0], pos[1] (ascending)
  unsigned char src[32];
  unsigned char dst[32];
};
static_assert(sizeof(TileOpDev) == 128, "TileOpDev layout");

// Where a diagonal op's table index comes from inside a tile, worked out by
// the planner; it overlays TileOpDev::src/dst of a diagonal op.  Index bit i
// is the table's qubit pos[i] (global, ascending): a tile bit (tpos[i]) or a
// qubit outside the tile, whose value is the same for the whole tile.  The
// in-tile bits are read as up to four runs, ((j >> run_t) & (2^run_n - 1))
// << run_i, or bit by bit (nruns = 255).  Required qubits are those whose 0
// value makes every entry exactly 1: inside the tile only the elements with
// them set are visited (req_t, ascending); outside it (out_req) a tile where
// one of them is 0 is left alone.
struct TileDiagInfo {
  unsigned char nruns;
  unsigned char nreq;
  unsigned short out_req;   // index bits of required qubits outside the tile
  unsigned char tpos[10];   // tile bit of index bit i, 255 outside the tile
  unsigned char run_t[4], run_n[4], run_i[4];
  unsigned char req_t[4];
};
static_assert(sizeof(TileDiagInfo) <= 64, "TileDiagInfo overlays src/dst");

// One stage of a tile pass (80 bytes): a register run or one shared-memory op.
struct TileStageDev {
  int reg;    // 1: register run of ops [first, first+count)
  int first;
  int count;
  int pad;
  int slots[6];   // tile bits of register slots, ascending
  int tpos[10];   // tile bits of thread-index bits, ascending
};
static_assert(sizeof(TileStageDev) == 80, "TileStageDev layout");

struct TileArgs {
  int t, L, nE, nops;
  int E[kTileMaxE];  // global qubit of tile bit L+e, ascending
  int ndata;         // complex elements of op data
  int kmax;          // widest dense/permutation op of the pass (1..5)
  int nstages;
  int R;             // register bits of the register stages (0: none)
  int tc;            // 1: the pass has tensor-core ops (kind 3)
  int pad;
  unsigned long long ntiles;
  int *status;       // device status word: set on a bounded wait that gave up
  const void *ops;     // TileOpDev[nops] in device memory
  const void *data;    // complex op data in device memory (state precision)
  const void *stages;  // TileStageDev[nstages] in device memory
  // diagonal tables in device memory, read in place: float2 entries (FP32)
  // or double-float pairs (FP64); a diagonal op's data is its entry offset
  const void *tables;
};

size_t tile_smem_bytes(int prec, int t, int L, int ndata, int nops, int nstages);
int launch_tile(qvmg_state s, const TileArgs &args);

}  // namespace qvmg
