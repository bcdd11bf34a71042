// plan.h -- host-side program representation, gate fusion and tile planning.
#pragma once
#include <stdint.h>

#include <complex>
#include <vector>

namespace qvmg {

using cd = std::complex<double>;

enum OpKind { OP_DENSE = 0, OP_DIAG = 1, OP_PERM = 2, OP_TC = 3 };

// Tensor-core tile ops: dense blocks of kTcMinQubits..kTcMaxQubits tile
// bits run as tcgen05 bf16x3 MMAs over chunks of 128 groups.
constexpr int kTcMinQubits = 3;
constexpr int kTcMaxQubits = 5;
constexpr int kTcRows = 128;

// One gate application (or fused block).  Qubits are in nat-tuple order:
// q[j] is bit j of the matrix index.
struct Op {
  int kind = OP_DENSE;
  std::vector<int> q;
  std::vector<cd> m;         // dense: D*D row-major; diag: D entries
  std::vector<int64_t> perm; // perm: D entries, new[j] = old[perm[j]]
  int k() const { return (int)q.size(); }
};

// Tile-local op: the unit of work inside a shared-memory tile pass.
struct TileOpHost {
  int kind;
  std::vector<int> pos;      // dense/perm/tc: tile-local bit positions (nat order)
                             // diag: global qubits (nat order)
  std::vector<cd> data;      // dense matrix, or diag table; tc: the split real
                             // form (tc_operand), two floats per element
  std::vector<int64_t> perm; // perm moves
};

// A stage of a tile pass: either a run of 1- and 2-qubit dense ops applied to
// amplitudes held in registers (each thread owns 2^R of them: the tile bits
// `slots`, R of them, ascending; the other tile bits index the thread), or a
// single op applied in shared memory.
struct TileStage {
  bool reg = false;
  int first = 0, count = 0;  // ops [first, first+count) of the pass
  std::vector<int> slots;    // register stage: tile bits of register slots 0..R-1
  std::vector<int> tpos;     // register stage: tile bits of thread-index bits, ascending
};

struct Pass {
  enum Kind { DENSE = 0, DIAG = 1, PERM = 2, TILE = 3 } kind;
  // DENSE / PERM: a single op (global qubits)
  Op op;
  // DIAG: tables (each over <= 10 global qubits)
  std::vector<std::vector<int>> tq;
  std::vector<std::vector<cd>> tables;
  // TILE
  int t = 0, L = 0;
  std::vector<int> E;  // global positions of tile bits L..t-1, ascending
  std::vector<TileOpHost> tops;
  int R = 0;           // register bits of the register stages (0: none)
  std::vector<TileStage> stages;
};

// Device descriptor sizes of tile ops and stages (tile.h), and the dynamic
// shared memory one tile pass may use (227 KiB per CTA on sm_103a, less 128
// bytes for the kernel's static shared variables).
constexpr size_t kTileOpDescBytes = 128;
constexpr size_t kTileStageDescBytes = 80;
constexpr size_t kTileSmemBudget = 227 * 1024 - 128;
// Tensor-core passes: two CTAs per SM share its 228 KiB (each also holding
// 1 KiB reserved by the runtime and its static variables).
constexpr size_t kTileSmemBudgetTc = 112 * 1024;
size_t tile_pass_smem_bytes(const Pass &p, int prec);

// Register bits per thread for a tile of t qubits run by 256 threads:
// FP32 tiles of 12 or 13 qubits hold 16 or 32 amplitudes per thread; other
// tiles (and FP64, whose 16-byte amplitudes would not fit) use shared memory.
int tile_register_bits(int prec, int t);
// Group a tile pass's ops into stages (register runs and shared-memory ops);
// canonicalises register ops so their slots ascend.
void build_stages(Pass &p, int prec, bool reg_stages);

struct Plan {
  int nq = -1, prec = -1, mode = -1, fw = -1, tile = -1;
  bool reg_stages = false;
  bool tensor_cores = false;
  std::vector<Pass> passes;
  int64_t n_src = 0, n_blocks = 0, n_tile = 0, n_diag = 0, n_perm = 0, n_dense = 0;
};

// Tensor-core operand of a dense k-qubit block (k = 3, 4): the real form
// Bt[n][kk] (n = 2r + re/im of output r, kk = 2c + re/im of input c), split
// into bf16 hi and lo parts (round to nearest even; lo = bf16(x - hi)),
// each laid out K-major in 8-row x 8-element core matrices: element (n, kk)
// at ((n/8)*(2D/8) + kk/8)*64 + (n%8)*8 + kk%8; hi block, then lo block.
std::vector<uint16_t> tc_operand(const std::vector<cd> &m, int k);
// Merge a tile pass's dense ops into blocks of at most `maxk` tile bits
// (moving an op past ops on disjoint qubits), then turn the blocks that fit
// the tensor-core path into OP_TC ops.
void merge_tile_ops(Pass &p, int maxk, bool tensor_cores);

// Gate fusion: merge consecutive gates into blocks of at most `fw` qubits.
std::vector<Op> fuse_ops(const std::vector<Op> &ops, int fw);
// Build a plan for a state of nq qubits.
void make_plan(const std::vector<Op> &ops, int nq, int prec, int mode, int fw, int tile,
               Plan &plan, bool reg_stages = false, bool tensor_cores = false);
// Default tile width (qubits held per tile) for a precision.
int default_tile_qubits(int prec);
int tile_low_bits(int prec);

}  // namespace qvmg
