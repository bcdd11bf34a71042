/*
 * qvm_oracle.h -- CPU oracle for the pure-state statevector path of the QVM.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * QVM's Lisp algorithms (quil-lang/qvm, src/wavefunction.lisp,
 * src/measurement.lisp, src/compile-gate.lisp, src/utilities.lisp,
 * src/linear-algebra.lisp, quil/stdgates.quil).  It is the checker that the
 * CUDA library's results are compared against, and the timed CPU baseline.
 * Nothing in the product (the qvm_gb300 package or libqvmgpu.so) links,
 * loads or calls it.
 *
 * Parity pinning: the reference is Common Lisp and cannot run here (no SBCL),
 * so this restatement is pinned against the known-answer tests the reference
 * ships in tests/gate-tests.lisp, tests/measurement-tests.lisp,
 * tests/linear-algebra-tests.lisp, tests/utilities-tests.lisp and
 * tests/wavefunction-tests.lisp (transcribed into tests/golden/).
 *
 * Layout: a wavefunction is 2^n complex doubles stored as interleaved
 * (re, im) doubles, amplitude index bit q = qubit q (LSB first), the layout
 * of the reference's (simple-array (complex double-float)).
 */
#ifndef QVM_ORACLE_H
#define QVM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* utilities.lisp:243-289 */
uint64_t orc_inject_bit(uint64_t x, int n);
uint64_t orc_eject_bit(uint64_t x, int n);
/* wavefunction.lisp:24-40 */
uint64_t orc_index_to_address(uint64_t index, int qubit, int state);
/* utilities.lisp:157-182; returns the number of ranges written */
int orc_subdivide(uint64_t total, int num_ranges, uint64_t *starts, uint64_t *ends);

/* Worker count and parallelisation threshold, the analogues of the
 * lparallel kernel size and *qubits-required-for-parallelization*
 * (config.lisp:14, default 19). */
void orc_set_workers(int workers);
int orc_get_workers(void);
void orc_set_parallel_threshold(int qubits);

/* wavefunction.lisp:80-109 */
void orc_bring_to_zero(double *wf, uint64_t len);
void orc_copy(const double *src, double *dst, uint64_t len);

/* wavefunction.lisp:44-70 */
double orc_ground_probability(const double *wf, int nq, int q);
double orc_excited_probability(const double *wf, int nq, int q);
/* wavefunction.lisp:332-364 */
double orc_norm(const double *wf, uint64_t len);
void orc_normalize(double *wf, uint64_t len, double length /* <=0: compute */);

/* wavefunction.lisp:271-330 + linear-algebra.lisp:97-131 (generic k).
 * qubits[] is a nat-tuple: qubits[0] is bit 0 of the matrix index, i.e. the
 * LAST qubit argument of the Quil gate application (utilities.lisp:43-51). */
void orc_apply_matrix_operator(double *wf, int nq, const double *matrix,
                               int k, const int *qubits);
/* compile-gate.lisp:259-309: amplitude j of each group becomes amplitude
 * perm[j] of the old group (out[j] = in[perm[j]]). */
void orc_apply_permutation(double *wf, int nq, int k, const int *qubits,
                           const int64_t *perm);
int orc_permutation_to_transpositions(int len, const int64_t *perm,
                                      int *left, int *right);

/* measurement.lisp:10-41 */
void orc_force_measurement(double *wf, int nq, int measured_value, int q,
                           double excited_probability);
/* measurement.lisp:87-105: returns the bit; *draw_used says whether the
 * uniform draw was consumed (it is not when p1 = 0). */
int orc_measure(double *wf, int nq, int q, double draw, int *draw_used,
                double *p1_out);
/* compile-gate.lisp:221-254: the compiled single-qubit measurement. */
int orc_measure_compiled(double *wf, int nq, int q, double draw,
                         double *p0_out);
/* measurement.lisp:179-225 */
uint64_t orc_sample_bisect(const double *wf, uint64_t len, double p);
/* measurement.lisp:128-143; returns the basis index */
uint64_t orc_measure_all(double *wf, int nq, double draw);
/* wavefunction.lisp:382-395 */
void orc_cdf(const double *wf, uint64_t len, double *cdf);
/* measurement.lisp:246-288, with caller-supplied draws */
void orc_sample_multiple(const double *wf, uint64_t len, const double *draws,
                         uint64_t nshots, uint64_t *out);
/* app/src/api/expectation.lisp:78-89: sum conj(a_i) b_i */
void orc_inner(const double *a, const double *b, uint64_t len, double *re,
               double *im);

/* Gate matrices of quil/stdgates.quil, row-major complex.  Returns 0 and
 * sets *k on success, -1 for an unknown name or wrong parameter count. */
int orc_gate_matrix(const char *name, const double *params, int nparams,
                    double *out, int *k);

#ifdef __cplusplus
}
#endif
#endif
