// plan.cpp -- gate fusion and shared-memory tile planning (host only).
//
// This is the GB300 counterpart of the reference's compile-loaded-program
// hook (src/qvm.lisp:166-175), which runs cl-quil's gate fusion
// (quil::fuse-gates-in-executable-code) and then specialises each gate
// (src/compile-gate.lisp:409-526).  The planner turns a gate list into
// device passes:
//
//  1. Fusion.  Gates are merged into dense blocks of at most `fw` qubits
//     when the merge is order-preserving: a gate joins a block that is the
//     latest op on all of the gate's qubits, or several blocks that are each
//     the latest op on all of their own qubits are merged with the gate.
//     Diagonal and permutation gates join a block only when that does not
//     widen it past two qubits (so a CPHASE chain stays a cheap phase op).
//  2. Tiling.  Each pass holds a tile of 2^t amplitudes in shared memory:
//     the low L qubits (a contiguous 2^L-amplitude row, L chosen so a row
//     is 256 bytes) plus up to t-L further qubits chosen greedily in
//     program order.  Every op whose mixing qubits lie in the tile is applied
//     in shared memory in that pass; diagonal ops need no tile membership
//     (their phase is read off the global amplitude index).  An op that
//     cannot join the pass blocks its qubits for the rest of the pass, which
//     keeps the op order on every qubit.
//  3. Diagonal runs are folded into phase tables over <= 10 qubits.
//  4. In FP32 plans for the tensor cores, each pass's dense ops are merged
//     into blocks of up to min(5, max(3, fw)) tile bits (an op may move past
//     ops on disjoint qubits), and the 3- to 5-qubit blocks become tcgen05
//     ops with their matrix split into bf16 hi and lo parts (merge_tile_ops).
#include "plan.h"

#include <algorithm>
#include <cstring>
#include <set>
#include <stdexcept>

#include "../../include/qvmgpu.h"

namespace qvmg {

static constexpr int kTableBits = 10;

int default_tile_qubits(int prec) { return prec == QVMG_FP64 ? 12 : 13; }
int tile_low_bits(int prec) { return prec == QVMG_FP64 ? 4 : 5; }

// Dense matrix of an op over its own qubits.
static std::vector<cd> op_matrix(const Op &op) {
  int d = 1 << op.k();
  if (op.kind == OP_DENSE) return op.m;
  std::vector<cd> m((size_t)d * d, cd(0, 0));
  if (op.kind == OP_DIAG) {
    for (int j = 0; j < d; ++j) m[(size_t)j * d + j] = op.m[j];
  } else {
    for (int j = 0; j < d; ++j) m[(size_t)j * d + op.perm[j]] = cd(1, 0);
  }
  return m;
}

// Embed the op's matrix into the qubit list `bq` (nat order), which must
// contain every op qubit.
static std::vector<cd> embed(const Op &op, const std::vector<int> &bq) {
  int kb = (int)bq.size();
  int db = 1 << kb;
  int k = op.k();
  std::vector<int> pos(k);
  for (int i = 0; i < k; ++i) {
    auto it = std::find(bq.begin(), bq.end(), op.q[i]);
    pos[i] = (int)(it - bq.begin());
  }
  unsigned mask = 0;
  for (int i = 0; i < k; ++i) mask |= 1u << pos[i];
  std::vector<cd> om = op_matrix(op);
  int d = 1 << k;
  std::vector<cd> out((size_t)db * db, cd(0, 0));
  for (int r = 0; r < db; ++r) {
    int rs = 0;
    for (int i = 0; i < k; ++i) rs |= ((r >> pos[i]) & 1) << i;
    for (int c = 0; c < db; ++c) {
      if ((r & ~mask) != (c & ~mask)) continue;
      int cs = 0;
      for (int i = 0; i < k; ++i) cs |= ((c >> pos[i]) & 1) << i;
      out[(size_t)r * db + c] = om[(size_t)rs * d + cs];
    }
  }
  return out;
}

static std::vector<cd> matmul(const std::vector<cd> &a, const std::vector<cd> &b, int d) {
  std::vector<cd> c((size_t)d * d, cd(0, 0));
  for (int i = 0; i < d; ++i)
    for (int l = 0; l < d; ++l) {
      cd x = a[(size_t)i * d + l];
      if (x == cd(0, 0)) continue;
      for (int j = 0; j < d; ++j) c[(size_t)i * d + j] += x * b[(size_t)l * d + j];
    }
  return c;
}

struct Unit {
  Op op;
  bool alive = true;
  bool block = false;  // a dense block open for merging
};

std::vector<Op> fuse_ops(const std::vector<Op> &ops, int fw) {
  std::vector<Unit> units;
  int maxq = 0;
  for (auto &op : ops)
    for (int q : op.q) maxq = std::max(maxq, q + 1);
  std::vector<int> latest(maxq, -1);

  auto is_latest_everywhere = [&](int u) {
    for (int q : units[u].op.q)
      if (latest[q] != u) return false;
    return true;
  };

  for (const Op &op : ops) {
    std::set<int> C;
    for (int q : op.q)
      if (latest[q] >= 0) C.insert(latest[q]);
    // Case A: the op lies inside one open block that is latest on its qubits.
    if (C.size() == 1) {
      int u = *C.begin();
      Unit &U = units[u];
      bool subset = true;
      for (int q : op.q)
        if (std::find(U.op.q.begin(), U.op.q.end(), q) == U.op.q.end()) subset = false;
      if (U.block && subset) {
        int db = 1 << U.op.k();
        U.op.m = matmul(embed(op, U.op.q), U.op.m, db);
        continue;
      }
    }
    // Case B: merge the op with the blocks that precede it on its qubits.
    int limit = op.kind == OP_DENSE ? fw : std::min(fw, 2);
    bool mergeable = op.k() <= limit;
    std::vector<int> bq;
    if (mergeable) {
      for (int u : C) {
        if (!units[u].block || !is_latest_everywhere(u)) {
          mergeable = false;
          break;
        }
        for (int q : units[u].op.q) bq.push_back(q);
      }
      for (int q : op.q)
        if (std::find(bq.begin(), bq.end(), q) == bq.end()) bq.push_back(q);
      if ((int)bq.size() > limit) mergeable = false;
    }
    if (mergeable && !C.empty()) {
      int db = 1 << (int)bq.size();
      std::vector<cd> acc((size_t)db * db, cd(0, 0));
      for (int i = 0; i < db; ++i) acc[(size_t)i * db + i] = cd(1, 0);
      for (int u : C) acc = matmul(embed(units[u].op, bq), acc, db);
      acc = matmul(embed(op, bq), acc, db);
      int last = *C.rbegin();
      for (int u : C)
        if (u != last) units[u].alive = false;
      Unit &U = units[last];
      U.op.kind = OP_DENSE;
      U.op.q = bq;
      U.op.m = acc;
      U.op.perm.clear();
      U.block = true;
      for (int q : bq) latest[q] = last;
      continue;
    }
    // Case C: a new unit.
    Unit nu;
    nu.op = op;
    nu.block = op.kind == OP_DENSE && op.k() <= fw;
    units.push_back(std::move(nu));
    int id = (int)units.size() - 1;
    for (int q : op.q) latest[q] = id;
  }
  std::vector<Op> out;
  for (auto &u : units)
    if (u.alive) out.push_back(std::move(u.op));
  return out;
}

// Group diagonal ops into phase tables of <= kTableBits qubits.
static void build_tables(const std::vector<const Op *> &diags,
                         std::vector<std::vector<int>> &tq,
                         std::vector<std::vector<cd>> &tables) {
  std::vector<std::vector<const Op *>> members;
  for (const Op *op : diags) {
    int best = -1;
    for (size_t t = 0; t < tq.size(); ++t) {
      std::set<int> u(tq[t].begin(), tq[t].end());
      for (int q : op->q) u.insert(q);
      if ((int)u.size() <= kTableBits) {
        best = (int)t;
        break;
      }
    }
    if (best < 0) {
      tq.push_back({});
      members.push_back({});
      best = (int)tq.size() - 1;
    }
    for (int q : op->q)
      if (std::find(tq[best].begin(), tq[best].end(), q) == tq[best].end())
        tq[best].push_back(q);
    members[best].push_back(op);
  }
  // ascending qubits: a table over a contiguous range of qubits is then
  // indexed by one shift and mask of the amplitude index
  for (auto &q : tq) std::sort(q.begin(), q.end());
  tables.resize(tq.size());
  for (size_t t = 0; t < tq.size(); ++t) {
    int kt = (int)tq[t].size();
    std::vector<cd> tab((size_t)1 << kt, cd(1, 0));
    for (const Op *op : members[t]) {
      std::vector<int> pos(op->k());
      for (int i = 0; i < op->k(); ++i)
        pos[i] = (int)(std::find(tq[t].begin(), tq[t].end(), op->q[i]) - tq[t].begin());
      for (int idx = 0; idx < (1 << kt); ++idx) {
        int s = 0;
        for (int i = 0; i < op->k(); ++i) s |= ((idx >> pos[i]) & 1) << i;
        tab[idx] *= op->m[s];
      }
    }
    tables[t] = std::move(tab);
  }
}

// Classify a dense op the way apply_dense does (permutation / diagonal).
static Op classify(const Op &op) {
  if (op.kind != OP_DENSE) return op;
  int d = 1 << op.k();
  bool diag = true, perm = true;
  std::vector<int64_t> p(d, -1);
  std::vector<int> seen(d, 0);
  for (int r = 0; r < d && (diag || perm); ++r) {
    int one = -1;
    for (int c = 0; c < d; ++c) {
      cd v = op.m[(size_t)r * d + c];
      if (r != c && v != cd(0, 0)) diag = false;
      if (v == cd(1, 0)) {
        if (one >= 0) perm = false;
        one = c;
      } else if (v != cd(0, 0)) {
        perm = false;
      }
    }
    if (one < 0 || seen[one]) perm = false;
    else { seen[one] = 1; p[r] = one; }
  }
  Op out = op;
  if (perm) {
    out.kind = OP_PERM;
    out.perm = p;
    out.m.clear();
  } else if (diag) {
    out.kind = OP_DIAG;
    std::vector<cd> dd(d);
    for (int j = 0; j < d; ++j) dd[j] = op.m[(size_t)j * d + j];
    out.m = dd;
  }
  return out;
}

static void emit_diag_passes(const std::vector<const Op *> &run, Plan &plan) {
  std::vector<std::vector<int>> tq;
  std::vector<std::vector<cd>> tables;
  build_tables(run, tq, tables);
  for (size_t t0 = 0; t0 < tq.size(); t0 += 4) {
    Pass p;
    p.kind = Pass::DIAG;
    for (size_t t = t0; t < std::min(tq.size(), t0 + 4); ++t) {
      p.tq.push_back(tq[t]);
      p.tables.push_back(tables[t]);
    }
    plan.passes.push_back(std::move(p));
    plan.n_diag++;
  }
}

static void plan_plain(const std::vector<Op> &ops, Plan &plan) {
  std::vector<Op> cls;
  cls.reserve(ops.size());
  for (auto &op : ops) cls.push_back(classify(op));
  std::vector<const Op *> run;
  for (size_t i = 0; i < cls.size(); ++i) {
    const Op &op = cls[i];
    if (op.kind == OP_DIAG) {
      run.push_back(&op);
      continue;
    }
    if (!run.empty()) {
      emit_diag_passes(run, plan);
      run.clear();
    }
    Pass p;
    p.kind = op.kind == OP_PERM ? Pass::PERM : Pass::DENSE;
    p.op = op;
    plan.passes.push_back(std::move(p));
    if (op.kind == OP_PERM) plan.n_perm++;
    else plan.n_dense++;
  }
  if (!run.empty()) emit_diag_passes(run, plan);
}

// Shared memory of a tile pass on the device: the tile, its row offsets
// (padded to 16 bytes), op data and op / stage descriptors (tile.h).
size_t tile_pass_smem_bytes(const Pass &p, int prec) {
  size_t csz = prec == QVMG_FP64 ? 16 : 8;
  size_t rows = (((size_t)1 << (p.t - p.L)) + 1) & ~(size_t)1;
  size_t b = ((size_t)1 << p.t) * csz + rows * 8;
  // (+ csz: a tensor-core operand starts on a 16-byte boundary)
  // (diagonal tables are read from global memory, not staged)
  for (auto &o : p.tops)
    b += (o.kind == OP_DIAG ? 0 : o.data.size() * csz) + kTileOpDescBytes +
         (o.kind == OP_TC ? csz : 0);
  b += p.stages.size() * kTileStageDescBytes;
  return (b + 15) & ~(size_t)15;
}

static void plan_fused(const std::vector<Op> &ops, int nq, int prec, int fw, int tile,
                       Plan &plan) {
  std::vector<Op> fused = fuse_ops(ops, fw);
  plan.n_blocks = (int64_t)fused.size();
  std::vector<Op> units;
  units.reserve(fused.size());
  for (auto &op : fused) units.push_back(classify(op));

  int L = std::min(tile_low_bits(prec), nq);
  int t = std::min(tile > 0 ? tile : default_tile_qubits(prec), nq);
  if (t < L + QVMG_MAX_GATE_QUBITS && t < nq) t = std::min(nq, L + QVMG_MAX_GATE_QUBITS);
  int cap = t - L;

  std::vector<int> remaining(units.size());
  for (size_t i = 0; i < units.size(); ++i) remaining[i] = (int)i;
  while (!remaining.empty()) {
    std::set<int> E, blocked;
    std::vector<int> in_pass, next;
    for (int u : remaining) {
      const Op &op = units[u];
      bool blk = false;
      for (int q : op.q)
        if (blocked.count(q)) blk = true;
      if (blk) {
        for (int q : op.q) blocked.insert(q);
        next.push_back(u);
        continue;
      }
      if (op.kind == OP_DIAG) {
        in_pass.push_back(u);
        continue;
      }
      std::set<int> hi;
      for (int q : op.q)
        if (q >= L && !E.count(q)) hi.insert(q);
      if ((int)(E.size() + hi.size()) <= cap) {
        E.insert(hi.begin(), hi.end());
        in_pass.push_back(u);
      } else {
        for (int q : op.q) blocked.insert(q);
        next.push_back(u);
      }
    }
    remaining.swap(next);
    bool all_diag = true;
    for (int u : in_pass)
      if (units[u].kind != OP_DIAG) all_diag = false;
    if (all_diag) {
      std::vector<const Op *> run;
      for (int u : in_pass) run.push_back(&units[u]);
      emit_diag_passes(run, plan);
      continue;
    }
    // Build the pass; if its shared-memory image (tile + op data +
    // descriptors) exceeds the per-CTA budget, hand the last ops back to the
    // next pass (a suffix in program order, so every qubit keeps its order).
    auto build_pass = [&](const std::vector<int> &members) {
      Pass p;
      p.kind = Pass::TILE;
      p.L = L;
      std::set<int> EE = E;
      // Fill the tile up to t qubits (unused tile bits cost nothing but keep
      // the tile geometry fixed): take the lowest qubits not yet in the tile.
      for (int q = L; q < nq && (int)EE.size() < cap; ++q) EE.insert(q);
      p.E.assign(EE.begin(), EE.end());
      p.t = L + (int)p.E.size();
      auto local = [&](int q) {
        if (q < L) return q;
        return L + (int)(std::find(p.E.begin(), p.E.end(), q) - p.E.begin());
      };
      std::vector<const Op *> drun;
      auto flush = [&]() {
        if (drun.empty()) return;
        std::vector<std::vector<int>> tq;
        std::vector<std::vector<cd>> tables;
        build_tables(drun, tq, tables);
        for (size_t i = 0; i < tq.size(); ++i) {
          TileOpHost top;
          top.kind = OP_DIAG;
          top.pos = tq[i];
          top.data = tables[i];
          p.tops.push_back(std::move(top));
        }
        drun.clear();
      };
      for (int u : members) {
        const Op &op = units[u];
        if (op.kind == OP_DIAG) {
          drun.push_back(&op);
          continue;
        }
        flush();
        TileOpHost top;
        top.kind = op.kind;
        for (int q : op.q) top.pos.push_back(local(q));
        if (op.kind == OP_DENSE) top.data = op.m;
        else top.perm = op.perm;
        p.tops.push_back(std::move(top));
      }
      flush();
      const bool tc = plan.tensor_cores && prec == QVMG_FP32;
      // tensor-core passes merge their dense ops into blocks of up to the
      // fusion width's qubits (3..5)
      if (tc) merge_tile_ops(p, std::min(kTcMaxQubits, std::max(kTcMinQubits, fw)), true);
      build_stages(p, prec, plan.reg_stages && !tc);
      return p;
    };
    Pass p = build_pass(in_pass);
    // a tensor-core pass keeps two CTAs per SM (one issues MMAs while the
    // other gathers): its shared memory stays within half an SM's
    const size_t budget =
        plan.tensor_cores && prec == QVMG_FP32 ? kTileSmemBudgetTc : kTileSmemBudget;
    while (tile_pass_smem_bytes(p, prec) > budget && in_pass.size() > 1) {
      remaining.insert(std::lower_bound(remaining.begin(), remaining.end(), in_pass.back()),
                       in_pass.back());
      in_pass.pop_back();
      p = build_pass(in_pass);
    }
    plan.passes.push_back(std::move(p));
    plan.n_tile++;
  }
}

// ---- tensor-core ops ---------------------------------------------------------------

// bf16 rounding of an FP32 value: round to nearest, ties to even (the
// device's cvt.rn.bf16.f32), as its 16-bit pattern.
static uint16_t bf16_rn(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

static double bf16_value(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return (double)f;
}

std::vector<uint16_t> tc_operand(const std::vector<cd> &m, int k) {
  const int D = 1 << k, N = 2 * D, K = 2 * D;
  std::vector<uint16_t> out((size_t)2 * N * K, 0);
  for (int n = 0; n < N; ++n)
    for (int kk = 0; kk < K; ++kk) {
      const int r = n >> 1, c = kk >> 1;
      const cd z = m[(size_t)r * D + c];
      double x;
      if ((n & 1) == 0) x = (kk & 1) == 0 ? z.real() : -z.imag();
      else x = (kk & 1) == 0 ? z.imag() : z.real();
      const uint16_t hi = bf16_rn((float)x);
      const uint16_t lo = bf16_rn((float)(x - bf16_value(hi)));
      const size_t idx = (size_t)((n >> 3) * (K >> 3) + (kk >> 3)) * 64 + (n & 7) * 8 + (kk & 7);
      out[idx] = hi;
      out[(size_t)N * K + idx] = lo;
    }
  return out;
}

// Global qubits an op of a tile pass touches.
static std::vector<int> op_globals(const Pass &p, const TileOpHost &o) {
  if (o.kind == OP_DIAG) return o.pos;
  std::vector<int> g;
  for (int b : o.pos) g.push_back(b < p.L ? b : p.E[b - p.L]);
  return g;
}

void merge_tile_ops(Pass &p, int maxk, bool tensor_cores) {
  std::vector<TileOpHost> out;
  for (TileOpHost &op : p.tops) {
    if (op.kind != OP_DENSE || (int)op.pos.size() > maxk) {
      out.push_back(std::move(op));
      continue;
    }
    const std::vector<int> g = op_globals(p, op);
    int target = -1;
    for (int i = (int)out.size() - 1; i >= 0; --i) {
      const TileOpHost &z = out[i];
      const std::vector<int> gz = op_globals(p, z);
      bool overlap = false;
      for (int q : g)
        if (std::find(gz.begin(), gz.end(), q) != gz.end()) overlap = true;
      if (z.kind == OP_DENSE) {
        std::set<int> u(z.pos.begin(), z.pos.end());
        u.insert(op.pos.begin(), op.pos.end());
        if ((int)u.size() <= maxk) {
          target = i;
          break;
        }
      }
      if (overlap) break;  // op cannot move before z
    }
    if (target < 0) {
      out.push_back(std::move(op));
      continue;
    }
    // z' = op . z over the union of their tile bits (op runs after z, and
    // commutes with every op between them)
    TileOpHost &z = out[target];
    std::vector<int> bq = z.pos;
    for (int b : op.pos)
      if (std::find(bq.begin(), bq.end(), b) == bq.end()) bq.push_back(b);
    Op oz, oo;
    oz.kind = oo.kind = OP_DENSE;
    oz.q = z.pos;
    oz.m = z.data;
    oo.q = op.pos;
    oo.m = op.data;
    const int db = 1 << (int)bq.size();
    z.data = matmul(embed(oo, bq), embed(oz, bq), db);
    z.pos = bq;
  }
  p.tops.swap(out);
  if (!tensor_cores) return;
  for (TileOpHost &op : p.tops) {
    const int k = (int)op.pos.size();
    if (op.kind != OP_DENSE || k < kTcMinQubits || k > kTcMaxQubits) continue;
    if ((1 << (p.t - k)) < kTcRows) continue;  // fewer than 128 groups
    // The bf16 operand travels as the bit patterns of FP32 values (two bf16
    // per float, the lower-addressed one in the low half): every such float
    // is finite, so the FP32 upload of the pass data copies it unchanged.
    const std::vector<uint16_t> h = tc_operand(op.data, k);
    op.kind = OP_TC;
    op.data.resize(h.size() / 4);
    for (size_t i = 0; i < op.data.size(); ++i) {
      const uint32_t w0 = (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 16);
      const uint32_t w1 = (uint32_t)h[4 * i + 2] | ((uint32_t)h[4 * i + 3] << 16);
      float f0, f1;
      std::memcpy(&f0, &w0, 4);
      std::memcpy(&f1, &w1, 4);
      op.data[i] = cd((double)f0, (double)f1);
    }
  }
}

int tile_register_bits(int prec, int t) {
  if (prec != QVMG_FP32) return 0;
  int r = t - 8;  // 256 threads
  return (r == 4 || r == 5) ? r : 0;
}

// Swap the matrix index bits of a 2-qubit op (so its qubit order flips).
static std::vector<cd> swap_2q(const std::vector<cd> &m) {
  auto sw = [](int i) { return ((i & 1) << 1) | ((i >> 1) & 1); };
  std::vector<cd> out(16);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[(size_t)sw(r) * 4 + sw(c)] = m[(size_t)r * 4 + c];
  return out;
}

void build_stages(Pass &p, int prec, bool reg_stages) {
  p.stages.clear();
  p.R = reg_stages ? tile_register_bits(prec, p.t) : 0;
  const int n = (int)p.tops.size();
  if (p.R == 0) {
    for (int i = 0; i < n; ++i) {
      TileStage s;
      s.first = i;
      s.count = 1;
      p.stages.push_back(s);
    }
    return;
  }
  auto reg_ok = [&](const TileOpHost &o) { return o.kind == OP_DENSE && o.pos.size() <= 2; };
  int i = 0;
  while (i < n) {
    if (!reg_ok(p.tops[i])) {
      TileStage s;
      s.first = i;
      s.count = 1;
      p.stages.push_back(s);
      ++i;
      continue;
    }
    // the longest run of register ops whose tile bits fit R slots
    std::set<int> bits;
    int j = i;
    while (j < n && reg_ok(p.tops[j])) {
      std::set<int> u = bits;
      u.insert(p.tops[j].pos.begin(), p.tops[j].pos.end());
      if ((int)u.size() > p.R) break;
      bits.swap(u);
      ++j;
    }
    TileStage s;
    s.reg = true;
    s.first = i;
    s.count = j - i;
    // pad the slots with the highest free tile bits, so that the thread bits
    // (the warp lanes) keep the low bits: consecutive lanes then touch
    // neighbouring shared-memory words
    for (int b = p.t - 1; b >= 0 && (int)bits.size() < p.R; --b) bits.insert(b);
    s.slots.assign(bits.begin(), bits.end());
    for (int b = 0; b < p.t; ++b)
      if (!bits.count(b)) s.tpos.push_back(b);
    // canonical qubit order: ascending slots (matrix index bit 0 = lower slot)
    for (int o = i; o < j; ++o) {
      TileOpHost &op = p.tops[o];
      if (op.pos.size() == 2 && op.pos[0] > op.pos[1]) {
        std::swap(op.pos[0], op.pos[1]);
        op.data = swap_2q(op.data);
      }
    }
    p.stages.push_back(s);
    i = j;
  }
}

void make_plan(const std::vector<Op> &ops, int nq, int prec, int mode, int fw, int tile,
               Plan &plan, bool reg_stages, bool tensor_cores) {
  plan = Plan();
  plan.reg_stages = reg_stages;
  plan.tensor_cores = tensor_cores;
  plan.nq = nq;
  plan.prec = prec;
  plan.mode = mode;
  plan.fw = fw;
  plan.tile = tile;
  plan.n_src = (int64_t)ops.size();
  if (mode == QVMG_RUN_PLAIN) plan_plain(ops, plan);
  else plan_fused(ops, nq, prec, fw, tile, plan);
}

}  // namespace qvmg
