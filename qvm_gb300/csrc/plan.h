// plan.h -- host-side program representation, gate fusion and tile planning.
#pragma once
#include <stdint.h>

#include <complex>
#include <vector>

namespace qvmg {

using cd = std::complex<double>;

enum OpKind { OP_DENSE = 0, OP_DIAG = 1, OP_PERM = 2 };

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
  std::vector<int> pos;      // dense/perm: tile-local bit positions (nat order)
                             // diag: global qubits (nat order)
  std::vector<cd> data;      // dense matrix, or diag table
  std::vector<int64_t> perm; // perm moves
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
};

struct Plan {
  int nq = -1, prec = -1, mode = -1, fw = -1, tile = -1;
  std::vector<Pass> passes;
  int64_t n_src = 0, n_blocks = 0, n_tile = 0, n_diag = 0, n_perm = 0, n_dense = 0;
};

// Gate fusion: merge consecutive gates into blocks of at most `fw` qubits.
std::vector<Op> fuse_ops(const std::vector<Op> &ops, int fw);
// Build a plan for a state of nq qubits.
void make_plan(const std::vector<Op> &ops, int nq, int prec, int mode, int fw, int tile,
               Plan &plan);
// Default tile width (qubits held per tile) for a precision.
int default_tile_qubits(int prec);
int tile_low_bits(int prec);

}  // namespace qvmg
