/*
 * qvmgpu.h -- C ABI of the GB300 (sm_103a) statevector engine for the QVM.
 *
 * This library is the drop-in replacement for the Lisp pure-state
 * representation of quil-lang/qvm.  A Lisp host (SBCL + CFFI) or any other
 * C-ABI caller owns opaque state handles whose amplitudes live in GPU HBM.
 * Every entry point below names the reference interface it replaces
 * (file:line in the quil-lang/qvm source tree).
 *
 * Conventions
 *  - Amplitude layout: index bit q = qubit q (LSB first).  Host buffers are
 *    complex128 (interleaved re, im doubles; 16 bytes per amplitude), the
 *    layout of the reference's (simple-array (complex double-float))
 *    (src/floats.lisp:13-27, scripts/shared_qvm.py:34-42).
 *  - Qubit tuples are nat-tuples (src/utilities.lisp:43-51): qubits[0] is
 *    bit 0 of the gate matrix's row/column index, i.e. the LAST argument of
 *    the Quil gate application "G a b" -> qubits = {b, a}.
 *  - Matrices are row-major 2^k x 2^k complex128.
 *  - Every function returns 0 (QVMG_OK) or a qvmg_status code; the message
 *    of the last failure on the calling thread is qvmg_last_error().
 *  - Random draws are supplied by the caller (the host keeps its MT19937
 *    stream and the reference's draw order), so results are reproducible.
 *  - Calls on one state are ordered on that state's own CUDA stream; calls
 *    on distinct states may run concurrently from different threads.
 */
#ifndef QVMGPU_H
#define QVMGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QVMG_ABI_VERSION 1
#define QVMG_MAX_QUBITS 34       /* 2^34 FP64 amplitudes = 256 GiB */
#define QVMG_MAX_GATE_QUBITS 5   /* per-op width of the dense/permutation ABI */
#define QVMG_MAX_DIAG_QUBITS 10  /* per-op width of the diagonal ABI */

typedef enum {
  QVMG_FP64 = 0, /* complex double: the reference's cflonum */
  QVMG_FP32 = 1  /* complex float: the fused split-precision form */
} qvmg_precision;

typedef enum {
  QVMG_OK = 0,
  QVMG_E_INVALID = 1,     /* bad argument (qubit out of range, bad k, ...) */
  QVMG_E_CUDA = 2,        /* a CUDA runtime call failed */
  QVMG_E_NOMEM = 3,       /* device allocation failed */
  QVMG_E_RANGE = 4,       /* probability out of range for a forced outcome */
  QVMG_E_UNSUPPORTED = 5, /* valid request this build does not handle */
  QVMG_E_TIMEOUT = 6      /* a bounded device-side wait gave up */
} qvmg_status;

typedef enum {
  /* src/measurement.lisp:87-105: p1 = P(q=1); no draw is consumed when
   * p1 = 0; otherwise bit = 1 iff draw <= p1. */
  QVMG_MEASURE_INTERPRETED = 0,
  /* src/compile-gate.lisp:221-254: p0 = P(q=0); the draw is always
   * consumed; bit = 0 iff draw < p0. */
  QVMG_MEASURE_COMPILED = 1
} qvmg_measure_convention;

typedef enum {
  /* src/measurement.lisp:179-225: smallest b with C(b) > p (len-1 if none). */
  QVMG_SAMPLE_BISECT = 0,
  /* src/measurement.lisp:246-288: smallest i with C(i) >= p (len-1 if none). */
  QVMG_SAMPLE_CDF = 1
} qvmg_sample_rule;

typedef enum {
  QVMG_RUN_PLAIN = 0, /* one pass per source gate, like apply-matrix-operator */
  QVMG_RUN_FUSED = 1  /* gate fusion + shared-memory tile passes */
} qvmg_run_mode;

typedef struct qvmg_state_s *qvmg_state;
typedef struct qvmg_program_s *qvmg_program;

/* ---- library ------------------------------------------------------------ */
const char *qvmg_last_error(void);
int qvmg_abi_version(void);
/* Device facts for admission control: SM count, free/total HBM bytes. */
int qvmg_device_info(int *sm_count, uint64_t *free_bytes, uint64_t *total_bytes);
/* Grow the device memory pool that states, scratch and plans come from by
 * `bytes` (in blocks of up to 16 GiB) and keep it: later allocations need no
 * new mapping, which can stall other threads' CUDA calls while the GPU is
 * busy.  A server calls it once with its HBM budget.  QVMG_E_NOMEM if the
 * device cannot hold it; then nothing stays reserved (the pool's unused memory
 * is returned to the device). */
int qvmg_device_reserve(uint64_t bytes);
/* Test hook (no counterpart in the reference, which has no device memory):
 * the `nth` device allocation the library makes from now on (1 = the next)
 * fails with QVMG_E_NOMEM without reaching CUDA; 0 cancels.  Lets host-side
 * tests drive the out-of-memory paths without exhausting a shared GPU. */
int qvmg_debug_fail_alloc(int nth);
/* Test hook (no counterpart in the reference): while `on` is 1, the warp that
 * issues a tensor-core tile op's MMAs issues none and commits nothing, so the
 * op's bounded wait runs out (in about a second): the run returns
 * QVMG_E_TIMEOUT, the kernel frees its tensor memory and the context stays
 * usable.  Lets tests drive the timeout path with nothing in flight. */
int qvmg_debug_tc_withhold(int on);
/* HBM bytes a state of this size and precision holds (16*2^n or 8*2^n plus
 * its reduction scratch); 0 for invalid arguments. */
uint64_t qvmg_state_bytes(int nqubits, int precision);

/* ---- state protocol (src/state-representation.lisp) ----------------------- */
/* make-pure-state :76-101 + allocate-vector (src/allocator.lisp:47-62):
 * allocate 2^n amplitudes in HBM set to |0...0>. */
int qvmg_state_create(int nqubits, int precision, qvmg_state *out);
/* The finalizer returned by allocate-vector (src/allocator.lisp:33-62). */
int qvmg_state_free(qvmg_state s);
/* num-qubits :138-140 */
int qvmg_state_info(qvmg_state s, int *nqubits, int *precision);
/* set-to-zero-state :150-152 -> bring-to-zero-state (src/wavefunction.lisp:80-91) */
int qvmg_state_reset(qvmg_state s);
/* (setf state-elements) :130-132: load 2^n complex128 amplitudes. */
int qvmg_state_upload(qvmg_state s, const double *amps);
/* state-elements :134-136 / amplitudes: read 2^n complex128 amplitudes. */
int qvmg_state_download(qvmg_state s, double *amps);
/* copy-wavefunction (src/wavefunction.lisp:93-109); both states must have
 * the same qubit count; precisions may differ (converted on the device). */
int qvmg_state_copy(qvmg_state dst, qvmg_state src);
/* Wait for all work queued on the state. */
int qvmg_state_sync(qvmg_state s);

/* ---- gate application (src/apply-gate.lisp:106-181) ---------------------- */
/* apply-matrix-operator (src/wavefunction.lisp:308-330) with the serial
 * kernels (src/serial-kernels.lisp:19-288): dense k-qubit matrix, k <= 5.
 * Diagonal and permutation matrices are routed to the kernels below, the
 * way compile-gate specialises constant matrices (src/compile-gate.lisp). */
int qvmg_apply_dense(qvmg_state s, int k, const int *qubits, const double *matrix);
/* Permutation gate (src/compile-gate.lisp:259-309): within each group,
 * new amplitude j = old amplitude perm[j]; k <= 5. */
int qvmg_apply_permutation(qvmg_state s, int k, const int *qubits, const int64_t *perm);
/* Diagonal gate (RZ, CPHASE, CZ, RZZ, PHASE, S, T ...): amplitude with
 * sub-index j is multiplied by diag[j] (2^k complex128); k <= 10. */
int qvmg_apply_diagonal(qvmg_state s, int k, const int *qubits, const double *diag);

/* ---- noise on pure states -------------------------------------------------- */
/* Reduced density matrix of k = 1 or 2 qubits: rho[r][c] (2^k x 2^k
 * complex128, row-major) = sum of a_r conj(a_c) over the other qubits, with
 * bit j of r <-> qubits[j].  Deterministic reduction order. */
int qvmg_reduced_density_matrix(qvmg_state s, int k, const int *qubits, double *rho);
/* %evolve-pure-state-stochastically (src/apply-gate.lisp:16-39): a Kraus map
 * of `nops` operators (each 2^k x 2^k complex128, row-major, stored one
 * after another) on k = 1 or 2 qubits.  Picks the first j whose running sum
 * of p_i = ||K_i psi||^2 reaches `draw` (the last operator if rounding
 * leaves the sum short), then replaces the state by K_j psi / sqrt(p_j).
 * *chosen and *probability (may be NULL) receive j and p_j.  QVMG_E_RANGE if
 * the selected p_j is zero. */
int qvmg_apply_kraus(qvmg_state s, int k, const int *qubits, int nops, const double *ops,
                     double draw, int *chosen, double *probability);
/* A density matrix of n qubits held as the 2n-qubit vector vec(rho), row
 * major (density-matrix-state, src/state-representation.lisp:173-266):
 * gates, Kraus maps (as the superoperator sum_j K_j (x) conj(K_j)),
 * measurement collapse and dephasing are ordinary 2n-qubit ops on it.  This
 * reads its diagonal: out[i] = Re rho[i][i] (2^n doubles), the outcome
 * distribution of density-matrix-state-measurement-probabilities
 * (src/state-representation.lisp:268-290). */
int qvmg_density_diagonal(qvmg_state s, double *out);

/* ---- measurement (src/measurement.lisp) ----------------------------------- */
/* wavefunction-excited-state-probability (src/wavefunction.lisp:62-70),
 * get-excited-state-probability (src/measurement.lisp:71-75); FP64 sum. */
int qvmg_prob_excited(qvmg_state s, int q, double *p1);
/* wavefunction-ground-state-probability (src/wavefunction.lisp:52-60) */
int qvmg_prob_ground(qvmg_state s, int q, double *p0);
/* force-measurement (src/measurement.lisp:10-41): zero the amplitudes with
 * bit q != bit and scale the rest by 1/sqrt(P(bit)), one pass. */
int qvmg_force_measurement(qvmg_state s, int q, int bit, double excited_probability);
/* measure (src/measurement.lisp:87-105) or the compiled measurement
 * (src/compile-gate.lisp:221-254): probability, draw, collapse.  *prob is
 * p1 (interpreted) or p0 (compiled); *draw_used is 0 when no draw was
 * consumed.  Any output pointer may be NULL. */
int qvmg_measure(qvmg_state s, int q, double draw, int convention, int *bit,
                 int *draw_used, double *prob);
/* measure-all-state (src/measurement.lisp:128-143): sample by the bisection
 * rule with one draw, then collapse to the basis state e_b (amplitude 1). */
int qvmg_measure_all(qvmg_state s, double draw, uint64_t *index);
/* Multishot sampling without collapse: one basis index per draw, by the
 * bisection rule (what repeated measure-all on a reloaded copy returns,
 * app/src/api/multishot-measure.lisp:93-109) or the CDF rule
 * (sample-wavefunction-multiple-times, src/measurement.lisp:246-288). */
int qvmg_sample(qvmg_state s, const double *draws, uint64_t nshots, int rule,
                uint64_t *out);
/* Multishot sampling that allocates nothing.  This entry point has no
 * counterpart in the reference: it serves callers that cannot allocate
 * device memory -- a host that owns the whole device pool and hands out
 * slices of it, or a latency-critical loop that cannot afford cudaMalloc's
 * implicit synchronisation -- and so cannot create a qvmg_state.  The caller
 * passes device pointers: `amps` (2^nqubits amplitudes, double2 for
 * QVMG_FP64 or float2 for QVMG_FP32, LSB-first), `draws` (nshots doubles in
 * [0, 1]) and `out` (nshots uint64 indices), plus the cudaStream_t to order
 * the work on (NULL = the default stream).  The call only queues work; the
 * results are in `out` once that stream reaches them.  Results equal
 * qvmg_sample's for the same amplitudes, draws and rule.
 *  - Limit: nqubits <= 30.  The CDF block sums live in a fixed 2 MiB device
 *    array (2^18 + 1 doubles) that every GPU which loads this library holds
 *    until the process exits; larger states are rejected with
 *    QVMG_E_INVALID.
 *  - The first call on a device looks up that array's device address (once
 *    per device); make that first call before any CUDA stream capture.
 *  - All calls share the one array.  Each call overwrites every entry it
 *    reads before reading it, but calls whose work overlaps on the GPU (on
 *    different streams, or from different threads) race on it: order them. */
int qvmg_sample_noalloc(const void *amps, int nqubits, int precision, const double *draws,
                        uint64_t nshots, int rule, uint64_t *out, void *stream);
/* |a_i|^2 for every amplitude (app/src/api/probabilities.lisp:13-19). */
int qvmg_probabilities(qvmg_state s, double *out);
/* Marginal distribution of k <= 20 distinct qubits: out[m] (2^k doubles) is
 * the sum of |a_i|^2 over the i whose bit qubits[j] equals bit j of m.  One
 * read of the state; the sums are deterministic (fixed reduction order). */
int qvmg_marginal_probabilities(qvmg_state s, int k, const int *qubits, double *out);
/* Repeated measurement of a resident state without collapsing it: the
 * trials of multishot-measure (app/src/api/multishot-measure.lisp:12-35,
 * 93-109), each of which reloads the prepared state and measures
 * qubits[0..k-1] in order with measure (src/measurement.lisp:87-105;
 * convention QVMG_MEASURE_INTERPRETED: a draw is taken only when p1 != 0,
 * bit = draw <= p1) or the compiled measurement
 * (src/compile-gate.lisp:221-254; QVMG_MEASURE_COMPILED: a draw every time,
 * bit = 0 iff draw < p0).  A qubit of -1 is an unused slot (bit 0, no draw);
 * a repeated qubit reads its earlier outcome.  At most 20 distinct qubits
 * (measuring every qubit is the measure-all path: qvmg_sample with
 * QVMG_SAMPLE_BISECT).  Draws are consumed in trial order, then list order;
 * bits[t*k + e] receives trial t, entry e; *draws_used the number consumed
 * (QVMG_E_RANGE when `ndraws` runs out).  The state is not modified. */
int qvmg_measure_sequence(qvmg_state s, int k, const int *qubits, int convention, int ntrials,
                          const double *draws, uint64_t ndraws, uint8_t *bits,
                          uint64_t *draws_used);
/* Wire bytes of the wavefunction endpoint (app/src/handle-request.lisp:
 * 132-152, write-complex-double-float-as-binary in app/src/utilities.lisp:
 * 62-77): per amplitude, the real then the imaginary part as IEEE doubles in
 * big-endian byte order; `out` holds 16 * 2^n octets. */
int qvmg_wavefunction_octets(qvmg_state s, uint8_t *out);
/* Wire bytes of the probabilities endpoint (app/src/handle-request.lisp:
 * 154-175, write-double-float-as-binary in app/src/utilities.lisp:79-87):
 * |a_i|^2 as big-endian IEEE doubles; `out` holds 8 * 2^n octets. */
int qvmg_probabilities_octets(qvmg_state s, uint8_t *out);
/* norm / normalize-wavefunction (src/wavefunction.lisp:332-364). */
int qvmg_norm(qvmg_state s, double *norm);
int qvmg_normalize(qvmg_state s);
/* inner product sum conj(a_i) b_i (app/src/api/expectation.lisp:80-84). */
int qvmg_inner(qvmg_state a, qvmg_state b, double *re, double *im);
/* |<a|b>|^2 / (<a|a><b|b>) and max_i |a_i - b_i| (precision report of the
 * fused form; the FP32 form is compared as a normalised state). */
int qvmg_fidelity(qvmg_state a, qvmg_state b, double *fidelity, double *max_abs_err);

/* ---- programs: transition loop over gate applications ------------------- */
/* A program is the gate-application part of a loaded Quil program
 * (src/classical-memory-mixin.lisp:114-159, src/execution.lisp:31-37), as a
 * list of ops.  QVMG_RUN_PLAIN applies them one pass per op (the
 * reference's transition -> apply-gate-to-state loop); QVMG_RUN_FUSED runs
 * them through the gate-fusion pass (the compile-loaded-program hook,
 * src/qvm.lisp:166-175) and shared-memory tile passes. */
int qvmg_program_create(qvmg_program *out);
int qvmg_program_free(qvmg_program p);
int qvmg_program_add_dense(qvmg_program p, int k, const int *qubits, const double *matrix);
/* n dense gates in one call: gate i has ks[i] qubits (nat-tuple order, packed
 * one after another in `qubits`) and a row-major 2^k x 2^k complex matrix
 * (packed in `matrices`).  Same validation as qvmg_program_add_dense; on an
 * invalid gate nothing is added. */
int qvmg_program_add_dense_many(qvmg_program p, int n, const int *ks, const int *qubits,
                                const double *matrices);
int qvmg_program_add_permutation(qvmg_program p, int k, const int *qubits, const int64_t *perm);
int qvmg_program_add_diagonal(qvmg_program p, int k, const int *qubits, const double *diag);
int qvmg_program_num_ops(qvmg_program p, int *nops);
/* Plan (host only, no GPU work): fusion width (max qubits of a fused block,
 * 1..QVMG_MAX_GATE_QUBITS) and tile width (qubits held per shared-memory
 * tile, 0 = default).  *npasses receives the number of device passes. */
int qvmg_program_plan(qvmg_program p, int nqubits, int precision, int mode,
                      int fusion_width, int tile_qubits, int *npasses);
/* Planner options (QVMG_OPT_*), kept with the program and used by the next
 * plan or run.  QVMG_OPT_REGISTER_STAGES: 1 = apply runs of 1-/2-qubit
 * blocks to amplitudes held in registers inside a tile (FP32, 12/13-qubit
 * tiles), 0 = every block through shared memory (default). */
#define QVMG_OPT_REGISTER_STAGES 1
/* QVMG_OPT_TENSOR_CORES: 1 = in FP32 tiles, merge each pass's dense blocks
 * into blocks of up to 4 qubits and run the 3- and 4-qubit ones on the
 * tensor cores (tcgen05 TF32 MMAs, operands split into hi + lo TF32 parts,
 * three products accumulated in FP32), 0 = CUDA-core FMAs (default). */
#define QVMG_OPT_TENSOR_CORES 2
int qvmg_program_set_option(qvmg_program p, int option, int value);
/* Plan statistics: stats[0]=source ops, [1]=passes, [2]=tile passes,
 * [3]=fused blocks, [4]=diagonal passes, [5]=permutation passes,
 * [6]=algorithmic bytes moved per run (2 x state bytes x passes),
 * [7]=bytes of op data and descriptors a run uploads to the device. */
int qvmg_program_plan_stats(qvmg_program p, int64_t *stats, int nstats);
/* JSON text of the last plan (passes, tile qubits, op data) for tools and
 * tests; *needed receives the buffer size required (with the NUL). */
int qvmg_program_plan_describe(qvmg_program p, char *buf, uint64_t cap, uint64_t *needed);
/* Run the program on the state (plans on first use for the state's size). */
int qvmg_program_run(qvmg_state s, qvmg_program p, int mode);
/* Same, recording a CUDA event around every pass on the state's stream;
 * waits for the run and writes each pass's device time (ms) and kind
 * (0 dense, 1 diagonal, 2 permutation, 3 tile) for up to `cap` passes. */
int qvmg_program_run_profiled(qvmg_state s, qvmg_program p, int mode, float *pass_ms,
                              int *pass_kind, int cap, int *npasses);
/* The cudaStream_t (as void*) the state's work is ordered on, so a caller
 * can order or time its own work against it. */
int qvmg_state_stream(qvmg_state s, void **stream);

/* Scheduling class of a state's work when several states share the GPU (the
 * serving engine; no reference counterpart, whose server runs one QVM per
 * connection thread, app/src/entry-point.lisp:655-673).
 *   1: the state's stream gets the device's highest stream priority, so the
 *      block scheduler starts its kernels' CTAs before those of other streams;
 *   0: default priority and grids (each tile pass one persistent CTA set);
 *  -1: default priority, and tile passes run as many short CTAs (16 tiles
 *      each) rather than persistent ones, so that high-priority work finds
 *      free SMs within a fraction of a millisecond.
 * Results do not depend on the class.  The state's queued work is finished
 * before its stream is replaced. */
int qvmg_state_set_priority(qvmg_state s, int priority);

/* ---- batched QAOA MaxCut instances -------------------------------------- */
/* Many uneven QAOA circuits (examples/qaoa.lisp:7-206: H on all qubits, then
 * p layers of ZZ(gamma) on every graph edge and RX(2 beta) on every qubit)
 * held as complex FP32 states and run in one persistent launch with a device
 * work queue, captured once as a CUDA graph.  The multishot sampling of
 * each result follows sample-wavefunction-multiple-times
 * (src/measurement.lisp:246-288) with caller-supplied draws.
 * edges: flat (u, v) pairs of all instances in order; nedges[i] per
 * instance; qubit counts 2..26; p <= 16; <= 64 edges per instance. */
typedef struct qvmg_qaoa_s *qvmg_qaoa_batch;
int qvmg_qaoa_batch_create(int ninst, const int *nqubits, const int *nedges, const int *edges,
                           int p, const double *gammas, const double *betas,
                           qvmg_qaoa_batch *out);
/* Replace the angles (ninst x p each) for the next run. */
int qvmg_qaoa_batch_set_angles(qvmg_qaoa_batch b, const double *gammas, const double *betas);
/* Run every instance: expectations[i] = <H_C> (FP64 sum of |a_x|^2 cut(x));
 * shots[i*nshots + t] = smallest x with C(x) >= draws[i*nshots + t]. */
int qvmg_qaoa_batch_run(qvmg_qaoa_batch b, const double *draws, int nshots,
                        double *expectations, uint32_t *shots);
/* Final state of one instance as complex128 (2^n values). */
int qvmg_qaoa_batch_state(qvmg_qaoa_batch b, int instance, double *amps);
/* Device bytes the batch holds. */
uint64_t qvmg_qaoa_batch_bytes(qvmg_qaoa_batch b);
int qvmg_qaoa_batch_free(qvmg_qaoa_batch b);

/* ---- batches of small programs (one persistent launch) ------------------- */
/* Many small, uneven programs run in one launch, each from |0...0> on its own
 * state: the per-request program runs of the reference's server
 * (app/src/api/multishot.lisp:87-101, app/src/handle-request.lisp) and
 * sample-wavefunction-multiple-times (src/measurement.lisp:246-288) for each
 * program.  Program i has nqubits[i] qubits (1..13 in QVMG_FP32, 1..12 in
 * QVMG_FP64), nops[i] dense gates and nshots[i] shots.  Gates are given in
 * order, all programs concatenated: op_k[] their widths (1..3), op_qubits[]
 * their nat-tuple qubits (k per gate), matrices[] their row-major 2^k x 2^k
 * complex matrices as interleaved doubles.  A program runs on one CTA, so its
 * results do not depend on the other programs of the batch. */
typedef struct qvmg_sbatch_s *qvmg_sbatch;
int qvmg_sbatch_create(int precision, int nprograms, const int *nqubits, const int *nops,
                       const int *op_k, const int *op_qubits, const double *matrices,
                       const int *nshots, qvmg_sbatch *out);
/* Run every program; draws (the programs' shots concatenated, each in [0, 1])
 * give the samples, written to shots[] as basis-state indices: the smallest i
 * with C(i) >= draw (FP32 states: draw times the state's total probability). */
int qvmg_sbatch_run(qvmg_sbatch b, const double *draws, uint64_t *shots);
/* Where program i's draws and shots start in the concatenated arrays. */
int qvmg_sbatch_shot_offset(qvmg_sbatch b, int program, uint64_t *offset);
/* Program i's final state as complex128 (after a run). */
int qvmg_sbatch_state(qvmg_sbatch b, int program, double *amps);
uint64_t qvmg_sbatch_bytes(qvmg_sbatch b);
int qvmg_sbatch_free(qvmg_sbatch b);

#ifdef __cplusplus
}
#endif
#endif
