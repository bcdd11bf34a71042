// internal.h -- shared definitions of the libqvmgpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/qvmgpu.h"

namespace qvmg {

// ---- errors -----------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define QVMG_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return ::qvmg::cuda_fail(_e, #call); \
  } while (0)

#define QVMG_CHECK_LAUNCH(what)                           \
  do {                                                    \
    cudaError_t _e = cudaGetLastError();                  \
    if (_e != cudaSuccess) return ::qvmg::cuda_fail(_e, what); \
  } while (0)

// ---- device-side result record of a measurement ------------------------------
struct MeasResult {
  double prob;      // p1 (interpreted) or p0 (compiled) or sum for norms
  double inv_norm;  // renormalisation factor of the kept half
  double aux;       // imaginary part / second reduction value
  double na, nb;    // squared norms of the two states of an inner product
  int bit;          // measured bit
  int draw_used;    // whether the draw was consumed
  unsigned long long index;  // measure-all index
  int status;       // device-side status (0 ok)
  int pad;
};

// Number of amplitudes whose |a|^2 sum forms one entry of the two-level CDF.
constexpr int kSampleBlockBits = 12;
// Fixed reduction grid: partial sums per reduction (deterministic order).
constexpr int kReduceBlocks = 1024;
constexpr int kReduceThreads = 256;

struct Program;

}  // namespace qvmg

struct qvmg_state_s {
  int nq = 0;
  int prec = QVMG_FP64;
  uint64_t len = 0;
  void *amps = nullptr;            // double2* or float2*
  cudaStream_t stream = nullptr;
  int device = 0;
  int priority = 0;                // qvmg_state_set_priority: -1 yield, 0 default, 1 high
  double *partials = nullptr;      // kReduceBlocks * 2 doubles
  double *block_sums = nullptr;    // 2^(n-kSampleBlockBits) (+1) doubles
  uint64_t nblocks = 0;
  qvmg::MeasResult *dres = nullptr;  // device result record
  qvmg::MeasResult *hres = nullptr;  // pinned host mirror
  void *staging = nullptr;         // device staging for precision conversion
  uint64_t staging_bytes = 0;
  void *pinned = nullptr;          // pinned host bounce buffer
  uint64_t pinned_bytes = 0;
  cudaEvent_t xfer_ev[2] = {nullptr, nullptr};  // pipelined device -> host transfers
  double *dvec = nullptr;          // device vector for draws / op tables
  uint64_t dvec_bytes = 0;
};

namespace qvmg {

inline uint64_t amp_bytes(int prec) { return prec == QVMG_FP64 ? 16 : 8; }

// Grid for a grid-stride loop over `work` items.
int grid_for(uint64_t work, int threads, int per_sm = 8);
int sm_count();

// Ensure state scratch buffers are large enough.
// Device memory of states, their scratch and uploaded plans comes from the
// stream-ordered allocator (cudaMallocAsync / cudaFreeAsync on the stream
// that uses it): a plain cudaFree waits for the whole device, which in the
// serving engine stalled every worker until all queued passes had drained.
// The device's default pool keeps freed memory for reuse.
int dev_alloc(void **p, size_t bytes, cudaStream_t s);
// True when the test hook qvmg_debug_fail_alloc asks this allocation to
// fail; every device allocation of the library consults it once.
bool alloc_fault_injected();
void dev_free(void *p, cudaStream_t s);
// A library stream for frees that must wait on other streams' events.
cudaStream_t free_stream();
int ensure_dvec(qvmg_state s, uint64_t bytes);
int ensure_staging(qvmg_state s, uint64_t bytes);
int ensure_pinned(qvmg_state s, uint64_t bytes);

// Pipelined device -> host transfer of `count` elements of `elem` bytes into
// `out`: chunk by chunk, produce(off, n, dst) queues on the state's stream
// the device work that writes elements [off, off+n) into device memory
// `dst` (the state's staging), or, when `produce` is null, the elements are
// the state's own amplitudes.  Chunks go through two pinned buffers; host
// threads copy chunk i-1 to `out` while chunk i is produced and copied.
using ProduceFn = int (*)(qvmg_state s, uint64_t off, uint64_t n, void *dst, void *ctx);
int stream_to_host(qvmg_state s, uint64_t count, size_t elem, void *out, ProduceFn produce,
                   void *ctx);

// One-time process-wide setup (kernel attributes and the like), safe when
// several threads make their first call at once: `setup` runs exactly once
// and every caller gets its result.
template <typename F>
cudaError_t once(std::once_flag &flag, cudaError_t &result, F &&setup) {
  std::call_once(flag, [&] { result = setup(); });
  return result;
}

// Validation helpers.
int check_state(qvmg_state s);
int check_qubits(qvmg_state s, int k, const int *qubits, int kmax);
// Make `waiter`'s stream wait for work queued so far on `producer`'s stream.
int order_states(qvmg_state waiter, qvmg_state producer);

// ---- kernels launched from other translation units -------------------------------
int launch_dense(qvmg_state s, int k, const int *qubits, const double *matrix);
int launch_permutation(qvmg_state s, int k, const int *qubits, const int64_t *perm);
int launch_diagonal(qvmg_state s, int k, const int *qubits, const double *diag);
// Diagonal table pass: ntables tables, table t holds 2^kt complex values
// (FP64 interleaved), its qubits in tq[t][0..kt-1] (nat order).
int launch_diag_tables(qvmg_state s, int ntables, const int *ks, const int *qubits,
                       const double *tables);
// Same, with the tables already in device memory in the state's precision.
int launch_diag_dev(qvmg_state s, int ntables, const int *ks, const int *qubits,
                    const void *dtables, int nreq, const int *req);
// Qubits every table holds whose 0 value makes every entry exactly 1 (at
// most 4, ascending); tables are interleaved (re, im) doubles.  Returns their
// count.
int diag_required_bits(int ntables, const int *ks, const int *qubits, const double *tables,
                       int *req);


}  // namespace qvmg
