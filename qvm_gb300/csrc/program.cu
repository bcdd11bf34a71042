// program.cu -- programs: the gate-application part of a loaded Quil program,
// planned (plan.cpp) and run pass by pass on a state's stream.
//
// QVMG_RUN_PLAIN reproduces the reference's transition loop: one device
// pass per source gate (src/execution.lisp:31-37 -> src/transition.lisp:
// 155-186 -> apply-gate-to-state), with diagonal runs folded into phase
// passes and permutation matrices moved as index remaps.  QVMG_RUN_FUSED
// runs the fused + tiled plan.
#include <cuda_runtime.h>

#include <cstddef>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "plan.h"
#include "tile.h"

namespace qvmg {

static_assert(sizeof(TileOpDev) == kTileOpDescBytes, "planner op descriptor size");
static_assert(sizeof(TileStageDev) == kTileStageDescBytes, "planner stage descriptor size");
static_assert(kTileMaxSmem == (int)kTileSmemBudget, "planner shared-memory budget");
static_assert(kTileTcRows == kTcRows, "tensor-core chunk rows");

// Device image of one plan for one precision.
struct DevicePlan {
  Plan plan;
  void *buf = nullptr;                  // op descriptors + data
  std::vector<size_t> pass_off;         // per pass: byte offset of its data
  std::vector<TileArgs> tile_args;      // per pass (TILE passes)
  std::vector<std::vector<int>> dks;    // per pass (DIAG passes): table widths
  std::vector<std::vector<int>> dqs;    // per pass (DIAG passes): flat qubits
  std::vector<std::vector<int>> dreq;   // per pass (DIAG passes): required qubits
  bool has_tc = false;                  // some tile pass runs tensor-core ops
  // Streams that ran this plan, each with an event recorded after its last
  // run: the buffer is freed in the library's free stream after all of them,
  // without waiting on the host.
  std::mutex use_mu;
  std::map<cudaStream_t, cudaEvent_t> uses;
  void note_use(cudaStream_t s) {
    std::lock_guard<std::mutex> g(use_mu);
    cudaEvent_t &ev = uses[s];
    if (!ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (ev) cudaEventRecord(ev, s);
  }
  ~DevicePlan() {
    cudaStream_t fs = free_stream();
    for (auto &u : uses) {
      if (u.second) {
        cudaStreamWaitEvent(fs, u.second, 0);
        cudaEventDestroy(u.second);
      }
    }
    if (buf) dev_free(buf, fs);
  }
};

}  // namespace qvmg

struct qvmg_program_s {
  std::vector<qvmg::Op> ops;
  std::mutex mu;
  // key: (nq, prec, mode, fw, tile, register stages, tensor cores)
  std::map<std::tuple<int, int, int, int, int, int, int>, std::unique_ptr<qvmg::DevicePlan>>
      plans;
  qvmg::Plan last_plan;  // most recent host-only plan (for statistics)
  int default_fw = 2;
  int default_tile = 0;
  int reg_stages = 0;
  int tensor_cores = 0;
};

namespace qvmg {

template <typename T>
static void put_complex(std::vector<unsigned char> &bytes, const std::vector<cd> &v) {
  size_t off = bytes.size();
  bytes.resize(off + v.size() * 2 * sizeof(T));
  T *p = reinterpret_cast<T *>(bytes.data() + off);
  for (size_t i = 0; i < v.size(); ++i) {
    p[2 * i] = (T)v[i].real();
    p[2 * i + 1] = (T)v[i].imag();
  }
}

static void align16(std::vector<unsigned char> &bytes) {
  while (bytes.size() % 16) bytes.push_back(0);
}

// A diagonal tile op's index layout inside its pass's tiles (TileDiagInfo):
// the tile bit of every table qubit, the in-tile bits as runs, and the
// required qubits (every table entry with one of them 0 is exactly 1).
static void fill_diag_info(TileOpDev &d, const TileOpHost &th, const Pass &ps) {
  TileDiagInfo info;
  std::memset(&info, 0, sizeof(info));
  const int k = (int)th.pos.size();
  for (int i = 0; i < k; ++i) {
    const int q = th.pos[i];
    int tp = 255;
    if (q < ps.L) tp = q;
    for (size_t e = 0; e < ps.E.size(); ++e)
      if (ps.E[e] == q) tp = ps.L + (int)e;
    info.tpos[i] = (unsigned char)tp;
  }
  // in-tile bits as runs of consecutive index bits on consecutive tile bits
  int nruns = 0;
  for (int i = 0; i < k;) {
    if (info.tpos[i] == 255) {
      ++i;
      continue;
    }
    int len = 1;
    while (i + len < k && info.tpos[i + len] != 255 && info.tpos[i + len] == info.tpos[i] + len)
      ++len;
    if (nruns < 4) {
      info.run_t[nruns] = info.tpos[i];
      info.run_n[nruns] = (unsigned char)len;
      info.run_i[nruns] = (unsigned char)i;
    }
    ++nruns;
    i += len;
  }
  info.nruns = nruns <= 4 ? (unsigned char)nruns : 255;
  // required qubits
  std::vector<int> req_t;
  for (int i = 0; i < k; ++i) {
    bool req = true;
    for (size_t e = 0; e < th.data.size() && req; ++e)
      if (!((e >> i) & 1) && th.data[e] != cd(1.0, 0.0)) req = false;
    if (!req) continue;
    if (info.tpos[i] == 255) info.out_req |= (unsigned short)(1u << i);
    else req_t.push_back(info.tpos[i]);
  }
  std::sort(req_t.begin(), req_t.end());
  if (req_t.size() > 4) req_t.resize(4);  // the rest are visited and skipped as unit
  info.nreq = (unsigned char)req_t.size();
  for (size_t r = 0; r < req_t.size(); ++r) info.req_t[r] = (unsigned char)req_t[r];
  std::memcpy(d.src, &info, sizeof(info));
}

static int build_device_plan(qvmg_program p, int nq, int prec, int mode, int fw, int tile,
                             DevicePlan &dp, cudaStream_t stream) {
  make_plan(p->ops, nq, prec, mode, fw, tile, dp.plan, p->reg_stages != 0,
            p->tensor_cores != 0);
  std::vector<unsigned char> bytes;
  const size_t csz = prec == QVMG_FP64 ? 16 : 8;
  dp.pass_off.assign(dp.plan.passes.size(), 0);
  dp.tile_args.assign(dp.plan.passes.size(), TileArgs{});
  dp.dks.assign(dp.plan.passes.size(), {});
  dp.dqs.assign(dp.plan.passes.size(), {});
  dp.dreq.assign(dp.plan.passes.size(), {});
  for (size_t i = 0; i < dp.plan.passes.size(); ++i) {
    const Pass &ps = dp.plan.passes[i];
    align16(bytes);
    dp.pass_off[i] = bytes.size();
    if (ps.kind == Pass::DIAG) {
      std::vector<double> flat;
      for (size_t t = 0; t < ps.tq.size(); ++t) {
        dp.dks[i].push_back((int)ps.tq[t].size());
        for (int q : ps.tq[t]) dp.dqs[i].push_back(q);
        if (prec == QVMG_FP64) put_complex<double>(bytes, ps.tables[t]);
        else put_complex<float>(bytes, ps.tables[t]);
        for (const cd &z : ps.tables[t]) {
          flat.push_back(z.real());
          flat.push_back(z.imag());
        }
      }
      int req[4];
      const int nreq = diag_required_bits((int)dp.dks[i].size(), dp.dks[i].data(),
                                          dp.dqs[i].data(), flat.data(), req);
      dp.dreq[i].assign(req, req + nreq);
    } else if (ps.kind == Pass::TILE) {
      TileArgs &ta = dp.tile_args[i];
      std::memset(&ta, 0, sizeof(ta));
      ta.t = ps.t;
      ta.L = ps.L;
      ta.nE = (int)ps.E.size();
      if (ta.nE > kTileMaxE) return fail(QVMG_E_UNSUPPORTED, "tile has too many qubits");
      for (int e = 0; e < ta.nE; ++e) ta.E[e] = ps.E[e];
      ta.nops = (int)ps.tops.size();
      ta.ntiles = 1ull << (nq - ps.t);
      // data first, then op descriptors
      std::vector<TileOpDev> descs(ps.tops.size());
      int ndata = 0;
      std::vector<cd> data;
      std::vector<cd> tables;  // diagonal tables: global memory, not shared
      for (size_t o = 0; o < ps.tops.size(); ++o) {
        const TileOpHost &th = ps.tops[o];
        TileOpDev &d = descs[o];
        std::memset(&d, 0, sizeof(d));
        d.kind = th.kind;
        d.k = (int)th.pos.size();
        for (int j = 0; j < d.k; ++j) d.pos[j] = th.pos[j];
        if (th.kind == OP_TC && (ndata & 1)) {  // 16-byte aligned operand
          data.push_back(cd(0, 0));
          ++ndata;
        }
        d.data = ndata;
        if (th.kind == OP_TC) {
          ta.tc = 1;
          dp.has_tc = true;
        }
        else if (th.kind != OP_DIAG) ta.kmax = std::max(ta.kmax, d.k);
        if (th.kind == OP_DIAG) {
          fill_diag_info(d, th, ps);
          d.data = (int)tables.size();
          tables.insert(tables.end(), th.data.begin(), th.data.end());
          continue;
        }
        if (th.kind == OP_PERM) {
          int nm = 0;
          for (size_t j = 0; j < th.perm.size(); ++j)
            if (th.perm[j] != (int64_t)j) {
              d.dst[nm] = (unsigned char)j;
              d.src[nm] = (unsigned char)th.perm[j];
              ++nm;
            }
          d.nmoved = nm;
        } else {
          data.insert(data.end(), th.data.begin(), th.data.end());
          ndata += (int)th.data.size();
        }
      }
      ta.ndata = ndata;
      if (ta.kmax == 0) ta.kmax = 1;  // diagonal-only tile
      // stages; register-stage ops carry their register slots
      ta.R = ps.R;
      std::vector<TileStageDev> sdev(ps.stages.size());
      for (size_t si = 0; si < ps.stages.size(); ++si) {
        const TileStage &st = ps.stages[si];
        TileStageDev &sd = sdev[si];
        std::memset(&sd, 0, sizeof(sd));
        sd.reg = st.reg ? 1 : 0;
        sd.first = st.first;
        sd.count = st.count;
        if (st.reg) {
          if ((int)st.slots.size() != ps.R || (int)st.tpos.size() != ps.t - ps.R ||
              st.tpos.size() > 10)
            return fail(QVMG_E_UNSUPPORTED, "register stage geometry out of range");
          for (size_t k = 0; k < st.slots.size(); ++k) sd.slots[k] = st.slots[k];
          for (size_t k = 0; k < st.tpos.size(); ++k) sd.tpos[k] = st.tpos[k];
          for (int o = st.first; o < st.first + st.count; ++o) {
            TileOpDev &d = descs[o];
            auto slot_of = [&](int b) {
              return (int)(std::find(st.slots.begin(), st.slots.end(), b) - st.slots.begin());
            };
            d.slot0 = slot_of(d.pos[0]);
            d.slot1 = d.k > 1 ? slot_of(d.pos[1]) : 0;
            if (d.slot0 >= ps.R || (d.k > 1 && (d.slot1 >= ps.R || d.slot1 <= d.slot0)))
              return fail(QVMG_E_UNSUPPORTED, "register op outside its stage's slots");
          }
        }
      }
      ta.nstages = (int)sdev.size();
      size_t data_off = bytes.size();
      if (prec == QVMG_FP64) put_complex<double>(bytes, data);
      else put_complex<float>(bytes, data);
      align16(bytes);
      size_t ops_off = bytes.size();
      bytes.resize(ops_off + descs.size() * sizeof(TileOpDev));
      std::memcpy(bytes.data() + ops_off, descs.data(), descs.size() * sizeof(TileOpDev));
      align16(bytes);
      size_t stages_off = bytes.size();
      bytes.resize(stages_off + sdev.size() * sizeof(TileStageDev));
      std::memcpy(bytes.data() + stages_off, sdev.data(), sdev.size() * sizeof(TileStageDev));
      align16(bytes);
      // Diagonal tables stay in global memory (read through the L1 cache):
      // staged in shared memory, a pass's tables (a CPHASE chain of a QFT
      // takes up to 3 x 1024 entries) left room for one CTA per SM.  FP64
      // plans hold them as double-float pairs, rounded on the host exactly as
      // the device rounds op data (hi = RN(x), lo = RN(x - hi)).
      size_t tables_off = bytes.size();
      if (prec == QVMG_FP64) {
        for (const cd &z : tables) {
          const float v[4] = {(float)z.real(), (float)(z.real() - (double)(float)z.real()),
                              (float)z.imag(), (float)(z.imag() - (double)(float)z.imag())};
          const size_t at = bytes.size();
          bytes.resize(at + sizeof(v));
          std::memcpy(bytes.data() + at, v, sizeof(v));
        }
      } else {
        put_complex<float>(bytes, tables);
      }
      // pointers are patched after upload
      ta.data = (const void *)data_off;
      ta.ops = (const void *)ops_off;
      ta.stages = (const void *)stages_off;
      ta.tables = (const void *)tables_off;
      if (tile_smem_bytes(prec, ta.t, ta.L, ta.ndata, ta.nops, ta.nstages) > (size_t)kTileMaxSmem)
        return fail(QVMG_E_UNSUPPORTED, "tile pass data exceeds shared memory");
    }
  }
  (void)csz;
  if (!bytes.empty()) {
    int rc = dev_alloc(&dp.buf, bytes.size(), stream);
    if (rc) return rc;
    // Upload on the state's stream and wait for it: a plain cudaMemcpy from
    // pageable memory may return before its DMA lands, and it is ordered on
    // the legacy default stream, which the state's non-blocking stream does
    // not wait for -- a kernel could read the descriptors before they arrive.
    QVMG_CUDA(cudaMemcpyAsync(dp.buf, bytes.data(), bytes.size(), cudaMemcpyHostToDevice,
                              stream));
    QVMG_CUDA(cudaStreamSynchronize(stream));
  }
  for (size_t i = 0; i < dp.plan.passes.size(); ++i) {
    if (dp.plan.passes[i].kind != Pass::TILE) continue;
    TileArgs &ta = dp.tile_args[i];
    ta.data = (const unsigned char *)dp.buf + (size_t)ta.data;
    ta.ops = (const unsigned char *)dp.buf + (size_t)ta.ops;
    ta.stages = (const unsigned char *)dp.buf + (size_t)ta.stages;
    ta.tables = (const unsigned char *)dp.buf + (size_t)ta.tables;
  }
  return QVMG_OK;
}

static int run_device_plan(qvmg_state s, DevicePlan &dp, cudaEvent_t *events = nullptr) {
  int rc = QVMG_OK;
  if (events) QVMG_CUDA(cudaEventRecord(events[0], s->stream));
  for (size_t i = 0; i < dp.plan.passes.size() && rc == QVMG_OK; ++i) {
    if (events && i > 0) QVMG_CUDA(cudaEventRecord(events[i], s->stream));
    const Pass &ps = dp.plan.passes[i];
    switch (ps.kind) {
      case Pass::DENSE: {
        std::vector<double> m(2 * ps.op.m.size());
        for (size_t j = 0; j < ps.op.m.size(); ++j) {
          m[2 * j] = ps.op.m[j].real();
          m[2 * j + 1] = ps.op.m[j].imag();
        }
        rc = launch_dense(s, ps.op.k(), ps.op.q.data(), m.data());
        break;
      }
      case Pass::PERM:
        rc = launch_permutation(s, ps.op.k(), ps.op.q.data(), ps.op.perm.data());
        break;
      case Pass::DIAG:
        rc = launch_diag_dev(s, (int)dp.dks[i].size(), dp.dks[i].data(), dp.dqs[i].data(),
                             (const unsigned char *)dp.buf + dp.pass_off[i],
                             (int)dp.dreq[i].size(), dp.dreq[i].data());
        break;
      case Pass::TILE: {
        TileArgs ta = dp.tile_args[i];
        ta.status = reinterpret_cast<int *>(reinterpret_cast<char *>(s->dres) +
                                            offsetof(MeasResult, status));
        rc = launch_tile(s, ta);
        break;
      }
    }
  }
  dp.note_use(s->stream);  // the plan's buffer is freed after this stream's passes
  if (dp.has_tc && rc == QVMG_OK) {
    // a tensor-core pass whose bounded MMA wait gave up has set the status word
    int *dstatus = reinterpret_cast<int *>(reinterpret_cast<char *>(s->dres) +
                                           offsetof(MeasResult, status));
    QVMG_CUDA(cudaMemcpyAsync(&s->hres->status, dstatus, sizeof(int), cudaMemcpyDeviceToHost,
                              s->stream));
    QVMG_CUDA(cudaStreamSynchronize(s->stream));
    if (s->hres->status != 0) {
      s->hres->status = 0;
      QVMG_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), s->stream));
      return fail(QVMG_E_TIMEOUT, "a tensor-core tile pass timed out waiting for its MMAs");
    }
  }
  if (events && rc == QVMG_OK)
    QVMG_CUDA(cudaEventRecord(events[dp.plan.passes.size()], s->stream));
  return rc;
}

static int check_op_qubits(int k, const int *qubits, int kmax) {
  if (k < 1 || k > kmax)
    return fail(QVMG_E_INVALID, "op width k=" + std::to_string(k) + " outside 1.." +
                                    std::to_string(kmax));
  if (!qubits) return fail(QVMG_E_INVALID, "null qubit tuple");
  for (int i = 0; i < k; ++i) {
    if (qubits[i] < 0 || qubits[i] >= QVMG_MAX_QUBITS)
      return fail(QVMG_E_INVALID, "qubit index " + std::to_string(qubits[i]) + " out of range");
    for (int j = 0; j < i; ++j)
      if (qubits[i] == qubits[j])
        return fail(QVMG_E_INVALID, "repeated qubit " + std::to_string(qubits[i]));
  }
  return QVMG_OK;
}

// JSON description of a plan: the passes, their qubits and op data.
static std::string describe_plan(const Plan &pl) {
  std::string s;
  char tmp[96];
  auto num = [&](double x) {
    snprintf(tmp, sizeof(tmp), "%.17g", x);
    s += tmp;
  };
  auto ints = [&](const std::vector<int> &v) {
    s += "[";
    for (size_t i = 0; i < v.size(); ++i) {
      if (i) s += ",";
      s += std::to_string(v[i]);
    }
    s += "]";
  };
  auto cplx = [&](const std::vector<cd> &v) {
    s += "[";
    for (size_t i = 0; i < v.size(); ++i) {
      if (i) s += ",";
      s += "[";
      num(v[i].real());
      s += ",";
      num(v[i].imag());
      s += "]";
    }
    s += "]";
  };
  auto i64s = [&](const std::vector<int64_t> &v) {
    std::vector<int> w(v.begin(), v.end());
    ints(w);
  };
  s += "{\"nq\":" + std::to_string(pl.nq) + ",\"passes\":[";
  for (size_t i = 0; i < pl.passes.size(); ++i) {
    const Pass &ps = pl.passes[i];
    if (i) s += ",";
    if (ps.kind == Pass::DENSE || ps.kind == Pass::PERM) {
      s += ps.kind == Pass::DENSE ? "{\"kind\":\"dense\",\"qubits\":" : "{\"kind\":\"perm\",\"qubits\":";
      ints(ps.op.q);
      if (ps.kind == Pass::DENSE) {
        s += ",\"matrix\":";
        cplx(ps.op.m);
      } else {
        s += ",\"perm\":";
        i64s(ps.op.perm);
      }
      s += "}";
    } else if (ps.kind == Pass::DIAG) {
      s += "{\"kind\":\"diag\",\"tables\":[";
      for (size_t t = 0; t < ps.tq.size(); ++t) {
        if (t) s += ",";
        s += "{\"qubits\":";
        ints(ps.tq[t]);
        s += ",\"table\":";
        cplx(ps.tables[t]);
        s += "}";
      }
      // the qubits the kernel requires set (it visits only those amplitudes)
      {
        std::vector<int> ks, qs;
        std::vector<double> flat;
        for (size_t t = 0; t < ps.tq.size(); ++t) {
          ks.push_back((int)ps.tq[t].size());
          qs.insert(qs.end(), ps.tq[t].begin(), ps.tq[t].end());
          for (const cd &z : ps.tables[t]) {
            flat.push_back(z.real());
            flat.push_back(z.imag());
          }
        }
        int req[4];
        const int nreq = diag_required_bits((int)ks.size(), ks.data(), qs.data(), flat.data(), req);
        s += "],\"req\":";
        ints(std::vector<int>(req, req + nreq));
        s += "}";
      }
    } else {
      s += "{\"kind\":\"tile\",\"t\":" + std::to_string(ps.t) + ",\"L\":" + std::to_string(ps.L) +
           ",\"E\":";
      ints(ps.E);
      s += ",\"R\":" + std::to_string(ps.R) + ",\"stages\":[";
      for (size_t si = 0; si < ps.stages.size(); ++si) {
        const TileStage &st = ps.stages[si];
        if (si) s += ",";
        s += "{\"reg\":" + std::to_string(st.reg ? 1 : 0) + ",\"first\":" +
             std::to_string(st.first) + ",\"count\":" + std::to_string(st.count) + ",\"slots\":";
        ints(st.slots);
        s += "}";
      }
      s += "]";
      s += ",\"ops\":[";
      for (size_t o = 0; o < ps.tops.size(); ++o) {
        const TileOpHost &th = ps.tops[o];
        if (o) s += ",";
        s += std::string("{\"kind\":\"") +
             (th.kind == OP_DENSE  ? "dense"
              : th.kind == OP_DIAG ? "diag"
              : th.kind == OP_TC   ? "tc"
                                   : "perm") +
             "\",\"pos\":";
        ints(th.pos);
        if (th.kind == OP_PERM) {
          s += ",\"perm\":";
          i64s(th.perm);
        } else {
          s += ",\"data\":";
          cplx(th.data);
        }
        if (th.kind == OP_DIAG) {
          // the index layout the kernel uses inside this pass's tiles
          TileOpDev d;
          std::memset(&d, 0, sizeof(d));
          fill_diag_info(d, th, ps);
          TileDiagInfo di;
          std::memcpy(&di, d.src, sizeof(di));
          std::vector<int> tpos(di.tpos, di.tpos + th.pos.size()), runs, req(di.req_t, di.req_t + di.nreq);
          if (di.nruns != 255)
            for (int r = 0; r < di.nruns; ++r) {
              runs.push_back(di.run_t[r]);
              runs.push_back(di.run_n[r]);
              runs.push_back(di.run_i[r]);
            }
          s += ",\"tpos\":";
          ints(tpos);
          s += ",\"nruns\":" + std::to_string(di.nruns) + ",\"runs\":";
          ints(runs);
          s += ",\"req_tile\":";
          ints(req);
          s += ",\"out_req\":" + std::to_string(di.out_req);
        }
        s += "}";
      }
      s += "]}";
    }
  }
  s += "]}";
  return s;
}

static int program_max_qubit(qvmg_program p) {
  int m = 0;
  for (auto &op : p->ops)
    for (int q : op.q) m = std::max(m, q + 1);
  return m;
}

}  // namespace qvmg

using namespace qvmg;

extern "C" {

int qvmg_program_create(qvmg_program *out) {
  if (!out) return fail(QVMG_E_INVALID, "null output handle");
  *out = new qvmg_program_s();
  return QVMG_OK;
}

int qvmg_program_free(qvmg_program p) {
  delete p;
  return QVMG_OK;
}

int qvmg_program_add_dense(qvmg_program p, int k, const int *qubits, const double *matrix) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  int rc = check_op_qubits(k, qubits, QVMG_MAX_GATE_QUBITS);
  if (rc) return rc;
  if (!matrix) return fail(QVMG_E_INVALID, "null matrix");
  Op op;
  op.kind = OP_DENSE;
  op.q.assign(qubits, qubits + k);
  int d = 1 << k;
  op.m.resize((size_t)d * d);
  for (int i = 0; i < d * d; ++i) op.m[i] = cd(matrix[2 * i], matrix[2 * i + 1]);
  std::lock_guard<std::mutex> g(p->mu);
  p->ops.push_back(std::move(op));
  p->plans.clear();
  return QVMG_OK;
}

int qvmg_program_add_dense_many(qvmg_program p, int n, const int *ks, const int *qubits,
                                const double *matrices) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  if (n < 0 || (n > 0 && (!ks || !qubits || !matrices)))
    return fail(QVMG_E_INVALID, "null gate arrays");
  std::vector<Op> ops;
  ops.reserve((size_t)n);
  size_t qoff = 0, moff = 0;
  for (int i = 0; i < n; ++i) {
    const int k = ks[i];
    int rc = check_op_qubits(k, qubits + qoff, QVMG_MAX_GATE_QUBITS);
    if (rc) return rc;
    Op op;
    op.kind = OP_DENSE;
    op.q.assign(qubits + qoff, qubits + qoff + k);
    const size_t d = (size_t)1 << k;
    op.m.resize(d * d);
    for (size_t j = 0; j < d * d; ++j) op.m[j] = cd(matrices[2 * (moff + j)], matrices[2 * (moff + j) + 1]);
    qoff += (size_t)k;
    moff += d * d;
    ops.push_back(std::move(op));
  }
  std::lock_guard<std::mutex> g(p->mu);
  for (auto &op : ops) p->ops.push_back(std::move(op));
  p->plans.clear();
  return QVMG_OK;
}

int qvmg_program_add_permutation(qvmg_program p, int k, const int *qubits, const int64_t *perm) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  int rc = check_op_qubits(k, qubits, QVMG_MAX_GATE_QUBITS);
  if (rc) return rc;
  if (!perm) return fail(QVMG_E_INVALID, "null permutation");
  int d = 1 << k;
  std::vector<int> seen(d, 0);
  for (int j = 0; j < d; ++j) {
    if (perm[j] < 0 || perm[j] >= d || seen[perm[j]])
      return fail(QVMG_E_INVALID, "not a permutation of 0..2^k-1");
    seen[perm[j]] = 1;
  }
  Op op;
  op.kind = OP_PERM;
  op.q.assign(qubits, qubits + k);
  op.perm.assign(perm, perm + d);
  std::lock_guard<std::mutex> g(p->mu);
  p->ops.push_back(std::move(op));
  p->plans.clear();
  return QVMG_OK;
}

int qvmg_program_add_diagonal(qvmg_program p, int k, const int *qubits, const double *diag) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  int rc = check_op_qubits(k, qubits, QVMG_MAX_DIAG_QUBITS);
  if (rc) return rc;
  if (!diag) return fail(QVMG_E_INVALID, "null diagonal");
  Op op;
  op.kind = OP_DIAG;
  op.q.assign(qubits, qubits + k);
  int d = 1 << k;
  op.m.resize(d);
  for (int i = 0; i < d; ++i) op.m[i] = cd(diag[2 * i], diag[2 * i + 1]);
  std::lock_guard<std::mutex> g(p->mu);
  p->ops.push_back(std::move(op));
  p->plans.clear();
  return QVMG_OK;
}

int qvmg_program_num_ops(qvmg_program p, int *nops) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  if (nops) *nops = (int)p->ops.size();
  return QVMG_OK;
}

int qvmg_program_plan(qvmg_program p, int nqubits, int precision, int mode, int fusion_width,
                      int tile_qubits, int *npasses) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  if (nqubits < 1 || nqubits > QVMG_MAX_QUBITS) return fail(QVMG_E_INVALID, "bad qubit count");
  if (precision != QVMG_FP64 && precision != QVMG_FP32)
    return fail(QVMG_E_INVALID, "bad precision");
  if (mode != QVMG_RUN_PLAIN && mode != QVMG_RUN_FUSED) return fail(QVMG_E_INVALID, "bad mode");
  if (fusion_width < 1 || fusion_width > QVMG_MAX_GATE_QUBITS)
    return fail(QVMG_E_INVALID, "fusion width must be 1..5");
  if (tile_qubits < 0 || tile_qubits > 16) return fail(QVMG_E_INVALID, "tile width must be 0..16");
  std::lock_guard<std::mutex> g(p->mu);
  if (program_max_qubit(p) > nqubits)
    return fail(QVMG_E_INVALID, "program uses a qubit beyond the state's qubit count");
  make_plan(p->ops, nqubits, precision, mode, fusion_width, tile_qubits, p->last_plan,
            p->reg_stages != 0, p->tensor_cores != 0);
  p->default_fw = fusion_width;
  p->default_tile = tile_qubits;
  if (npasses) *npasses = (int)p->last_plan.passes.size();
  return QVMG_OK;
}

int qvmg_program_set_option(qvmg_program p, int option, int value) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  std::lock_guard<std::mutex> g(p->mu);
  if (option == QVMG_OPT_TENSOR_CORES) {
    if (value != 0 && value != 1) return fail(QVMG_E_INVALID, "tensor-core option is 0 or 1");
    p->tensor_cores = value;
    return QVMG_OK;
  }
  if (option == QVMG_OPT_REGISTER_STAGES) {
    if (value != 0 && value != 1) return fail(QVMG_E_INVALID, "register stages option is 0 or 1");
    p->reg_stages = value;
    return QVMG_OK;
  }
  return fail(QVMG_E_INVALID, "unknown program option " + std::to_string(option));
}

int qvmg_program_plan_stats(qvmg_program p, int64_t *stats, int nstats) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  const Plan &pl = p->last_plan;
  int64_t state_bytes = pl.nq > 0 ? ((int64_t)1 << pl.nq) * (pl.prec == QVMG_FP64 ? 16 : 8) : 0;
  // bytes a run uploads when it builds its device plan
  int64_t csz = pl.prec == QVMG_FP64 ? 16 : 8, up = 0;
  for (const Pass &ps : pl.passes) {
    if (ps.kind == Pass::DIAG)
      for (auto &t : ps.tables) up += csz * (int64_t)t.size();
    if (ps.kind == Pass::TILE)
      for (auto &o : ps.tops) up += csz * (int64_t)o.data.size() + (int64_t)sizeof(TileOpDev);
  }
  int64_t v[8] = {pl.n_src, (int64_t)pl.passes.size(), pl.n_tile, pl.n_blocks, pl.n_diag,
                  pl.n_perm, 2 * state_bytes * (int64_t)pl.passes.size(), up};
  for (int i = 0; i < nstats && i < 8; ++i) stats[i] = v[i];
  return QVMG_OK;
}

int qvmg_program_plan_describe(qvmg_program p, char *buf, uint64_t cap, uint64_t *needed) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  std::string js = describe_plan(p->last_plan);
  if (needed) *needed = js.size() + 1;
  if (buf && cap > 0) {
    size_t n = std::min<size_t>(cap - 1, js.size());
    std::memcpy(buf, js.data(), n);
    buf[n] = 0;
    if (n < js.size()) return fail(QVMG_E_INVALID, "buffer too small for the plan description");
  }
  return QVMG_OK;
}

// Find or build the device plan of `p` for state `s` (caller holds p->mu).
static int device_plan_for(qvmg_state s, qvmg_program p, int mode, DevicePlan **out) {
  int rc = check_state(s);
  if (rc) return rc;
  if (!p) return fail(QVMG_E_INVALID, "null program");
  if (mode != QVMG_RUN_PLAIN && mode != QVMG_RUN_FUSED) return fail(QVMG_E_INVALID, "bad mode");
  if (program_max_qubit(p) > s->nq)
    return fail(QVMG_E_INVALID, "program uses a qubit beyond the state's qubit count");
  int fw = mode == QVMG_RUN_FUSED ? p->default_fw : 1;
  int tile = mode == QVMG_RUN_FUSED ? p->default_tile : 0;
  auto key = std::make_tuple(s->nq, s->prec, mode, fw, tile, p->reg_stages, p->tensor_cores);
  auto it = p->plans.find(key);
  if (it == p->plans.end()) {
    auto dp = std::make_unique<DevicePlan>();
    if ((rc = build_device_plan(p, s->nq, s->prec, mode, fw, tile, *dp, s->stream))) return rc;
    it = p->plans.emplace(key, std::move(dp)).first;
  }
  *out = it->second.get();
  return QVMG_OK;
}

int qvmg_program_run(qvmg_state s, qvmg_program p, int mode) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  std::lock_guard<std::mutex> g(p->mu);
  DevicePlan *dp = nullptr;
  int rc = device_plan_for(s, p, mode, &dp);
  if (rc) return rc;
  return run_device_plan(s, *dp);
}

int qvmg_program_run_profiled(qvmg_state s, qvmg_program p, int mode, float *pass_ms,
                              int *pass_kind, int cap, int *npasses) {
  if (!p) return fail(QVMG_E_INVALID, "null program");
  std::lock_guard<std::mutex> g(p->mu);
  DevicePlan *dp = nullptr;
  int rc = device_plan_for(s, p, mode, &dp);
  if (rc) return rc;
  size_t np = dp->plan.passes.size();
  std::vector<cudaEvent_t> ev(np + 1);
  for (auto &e : ev) QVMG_CUDA(cudaEventCreate(&e));
  rc = run_device_plan(s, *dp, ev.data());
  if (rc == QVMG_OK) {
    cudaError_t e = cudaEventSynchronize(ev[np]);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventSynchronize");
  }
  if (rc == QVMG_OK) {
    for (size_t i = 0; i < np && (int)i < cap; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      if (pass_ms) pass_ms[i] = ms;
      if (pass_kind) pass_kind[i] = (int)dp->plan.passes[i].kind;
    }
    if (npasses) *npasses = (int)np;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  return rc;
}

int qvmg_state_stream(qvmg_state s, void **stream) {
  int rc = check_state(s);
  if (rc) return rc;
  if (stream) *stream = (void *)s->stream;
  return QVMG_OK;
}

}  // extern "C"
