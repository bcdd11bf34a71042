/*
 * qvm_oracle.c -- CPU oracle (test infrastructure) for the QVM pure-state
 * statevector path.  See qvm_oracle.h for scope and parity pinning.
 *
 * Each function names the reference file:line it restates.  Arithmetic
 * follows the reference's expression order and is compiled without FMA
 * contraction (-ffp-contract=off), the way SBCL evaluates double-float
 * complex arithmetic: (a+bi)(c+di) = (ac-bd) + (ad+bc)i.
 *
 * Parallelism mirrors the reference's lparallel usage: loops over 2^n
 * amplitudes run on orc_get_workers() OpenMP threads once the qubit count
 * reaches the parallelisation threshold (config.lisp:14), and parallel sums
 * add per-range partial sums over subdivide(total, workers)
 * (utilities.lisp:395-425) in range order.
 */
#include "qvm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_workers = 1;
static int g_threshold = 19; /* *qubits-required-for-parallelization* */

void orc_set_workers(int workers) { g_workers = workers < 1 ? 1 : workers; }
int orc_get_workers(void) { return g_workers; }
void orc_set_parallel_threshold(int qubits) { g_threshold = qubits; }

/* utilities.lisp:243-255 (inject-bit) */
uint64_t orc_inject_bit(uint64_t x, int n) {
  uint64_t low_mask = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
  uint64_t left = (x & ~low_mask) << 1;
  uint64_t right = x & low_mask;
  return left | right;
}

/* utilities.lisp:267-279 (eject-bit) */
uint64_t orc_eject_bit(uint64_t x, int n) {
  uint64_t low_mask = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
  uint64_t left = (x >> 1) & ~low_mask;
  uint64_t right = x & low_mask;
  return left | right;
}

/* wavefunction.lisp:24-40 (index-to-address) */
uint64_t orc_index_to_address(uint64_t index, int qubit, int state) {
  uint64_t a = orc_inject_bit(index, qubit);
  if (state) a |= (1ull << qubit);
  return a;
}

/* utilities.lisp:157-182 (map-subdivisions / subdivide) */
int orc_subdivide(uint64_t total, int num_ranges, uint64_t *starts,
                  uint64_t *ends) {
  uint64_t size = total / (uint64_t)num_ranges;
  if (size == 0) {
    starts[0] = 0;
    ends[0] = total;
    return 1;
  }
  uint64_t start = 0;
  for (int w = 1; w <= num_ranges; ++w, start += size) {
    starts[w - 1] = start;
    ends[w - 1] = (w == num_ranges) ? total : start + size;
  }
  return num_ranges;
}

static int parallel_p(uint64_t count) {
  /* psum-dotimes / with-parallel-subdivisions: parallel when the count is
   * at least 2^threshold (utilities.lisp:356,400). */
  return g_workers > 1 && g_threshold < 63 && count >= (1ull << g_threshold);
}

static inline double prob(const double *wf, uint64_t i) {
  /* wavefunction.lisp:44-50 */
  double re = wf[2 * i], im = wf[2 * i + 1];
  return re * re + im * im;
}

/* A generic psum-dotimes over [0, range) whose body maps i -> prob(addr(i)).
 * kind 0: contiguous from base; 1: ground state of qubit q; 2: excited. */
typedef struct {
  const double *wf;
  uint64_t base;
  int kind;
  int q;
} sum_body;

static inline double body_eval(const sum_body *b, uint64_t i) {
  switch (b->kind) {
    case 1: return prob(b->wf, orc_inject_bit(i, b->q));
    case 2: return prob(b->wf, orc_index_to_address(i, b->q, 1));
    default: return prob(b->wf, b->base + i);
  }
}

static double psum_dotimes(const sum_body *b, uint64_t range) {
  if (!parallel_p(range)) {
    double s = 0.0;
    for (uint64_t i = 0; i < range; ++i) s += body_eval(b, i);
    return s;
  }
  int nw = g_workers;
  uint64_t *starts = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  uint64_t *ends = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  double *parts = (double *)calloc(nw, sizeof(double));
  int nr = orc_subdivide(range, nw, starts, ends);
#pragma omp parallel for num_threads(nw) schedule(static, 1)
  for (int r = 0; r < nr; ++r) {
    double s = 0.0;
    for (uint64_t i = starts[r]; i < ends[r]; ++i) s += body_eval(b, i);
    parts[r] = s;
  }
  double total = 0.0;
  for (int r = 0; r < nr; ++r) total += parts[r];
  free(starts);
  free(ends);
  free(parts);
  return total;
}

/* wavefunction.lisp:80-91 (bring-to-zero-state) */
void orc_bring_to_zero(double *wf, uint64_t len) {
  int par = parallel_p(len);
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t i = 0; i < (int64_t)(2 * len); ++i) wf[i] = 0.0;
  wf[0] = 1.0;
}

/* wavefunction.lisp:93-109 (copy-wavefunction) */
void orc_copy(const double *src, double *dst, uint64_t len) {
  int par = parallel_p(len);
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t i = 0; i < (int64_t)(2 * len); ++i) dst[i] = src[i];
}

/* wavefunction.lisp:52-60 */
double orc_ground_probability(const double *wf, int nq, int q) {
  sum_body b = {wf, 0, 1, q};
  return psum_dotimes(&b, (1ull << nq) / 2);
}

/* wavefunction.lisp:62-70 */
double orc_excited_probability(const double *wf, int nq, int q) {
  sum_body b = {wf, 0, 2, q};
  return psum_dotimes(&b, (1ull << nq) / 2);
}

/* wavefunction.lisp:332-346 (norm: psum over all amplitudes) */
double orc_norm(const double *wf, uint64_t len) {
  sum_body b = {wf, 0, 0, 0};
  return sqrt(psum_dotimes(&b, len));
}

/* wavefunction.lisp:349-364 */
void orc_normalize(double *wf, uint64_t len, double length) {
  double inv = 1.0 / (length > 0.0 ? length : orc_norm(wf, len));
  int par = len > (1ull << g_threshold) && g_workers > 1; /* pdotimes */
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t i = 0; i < (int64_t)len; ++i) {
    wf[2 * i] = inv * wf[2 * i];
    wf[2 * i + 1] = inv * wf[2 * i + 1];
  }
}

/* wavefunction.lisp:112-122 (set-qubit-components-of-amplitude-address) */
static inline uint64_t set_components(uint64_t address, uint64_t flags,
                                      const int *qubits, int k) {
  for (int j = 0; j < k; ++j) {
    uint64_t bit = 1ull << qubits[j];
    if (flags & 1ull) address |= bit; else address &= ~bit;
    flags >>= 1;
  }
  return address;
}

static int cmp_int(const void *a, const void *b) {
  return (*(const int *)a) - (*(const int *)b);
}

/* wavefunction.lisp:155-175 (map-complement) + :234-269
 * (with-modified-amplitudes) + :271-306 (apply-operator) + :308-330
 * (apply-matrix-operator) + linear-algebra.lisp:97-131 (matrix-multiply).
 * The serial 1q/2q/3q kernels (serial-kernels.lisp:19-168) compute the same
 * sums in the same order, so one generic routine covers every branch. */
void orc_apply_matrix_operator(double *wf, int nq, const double *m, int k,
                               const int *qubits) {
  int sorted[64];
  memcpy(sorted, qubits, sizeof(int) * k);
  qsort(sorted, k, sizeof(int), cmp_int);
  uint64_t dim = 1ull << k;
  uint64_t groups = 1ull << (nq - k);
  int par = parallel_p(1ull << nq) && nq >= g_threshold;
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t gi = 0; gi < (int64_t)groups; ++gi) {
    double col_re[64], col_im[64], res_re[64], res_im[64];
    double *cr = col_re, *ci = col_im, *rr = res_re, *ri = res_im;
    double *heap = NULL;
    if (dim > 64) {
      heap = (double *)malloc(sizeof(double) * 4 * dim);
      cr = heap; ci = heap + dim; rr = heap + 2 * dim; ri = heap + 3 * dim;
    }
    uint64_t j = (uint64_t)gi;
    for (int s = 0; s < k; ++s) j = orc_inject_bit(j, sorted[s]);
    for (uint64_t c = 0; c < dim; ++c) { /* extract */
      uint64_t a = set_components(j, c, qubits, k);
      cr[c] = wf[2 * a];
      ci[c] = wf[2 * a + 1];
    }
    for (uint64_t r = 0; r < dim; ++r) { /* matrix-multiply */
      double er = 0.0, ei = 0.0;
      for (uint64_t c = 0; c < dim; ++c) {
        double mr = m[2 * (r * dim + c)], mi = m[2 * (r * dim + c) + 1];
        double pr = mr * cr[c] - mi * ci[c];
        double pi = mr * ci[c] + mi * cr[c];
        er = er + pr;
        ei = ei + pi;
      }
      rr[r] = er;
      ri[r] = ei;
    }
    for (uint64_t c = 0; c < dim; ++c) { /* insert */
      uint64_t a = set_components(j, c, qubits, k);
      wf[2 * a] = rr[c];
      wf[2 * a + 1] = ri[c];
    }
    free(heap);
  }
}

/* compile-gate.lisp:259-268 (permutation-to-transpositions) */
int orc_permutation_to_transpositions(int len, const int64_t *perm, int *left,
                                      int *right) {
  int n = 0;
  for (int dest = 0; dest < len; ++dest) {
    int64_t src = perm[dest];
    while (src < dest) src = perm[src];
    if (src != dest) {
      left[n] = (int)src;
      right[n] = dest;
      ++n;
    }
  }
  return n;
}

/* compile-gate.lisp:270-309: complement iteration, then ROTATEF of the
 * addressed amplitudes for each transposition in order. */
void orc_apply_permutation(double *wf, int nq, int k, const int *qubits,
                           const int64_t *perm) {
  int len = 1 << k;
  int *left = (int *)malloc(sizeof(int) * len);
  int *right = (int *)malloc(sizeof(int) * len);
  int nt = orc_permutation_to_transpositions(len, perm, left, right);
  int sorted[64];
  memcpy(sorted, qubits, sizeof(int) * k);
  qsort(sorted, k, sizeof(int), cmp_int);
  uint64_t groups = 1ull << (nq - k);
  int par = parallel_p(groups);
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t gi = 0; gi < (int64_t)groups; ++gi) {
    uint64_t base = (uint64_t)gi;
    for (int s = 0; s < k; ++s) base = orc_inject_bit(base, sorted[s]);
    for (int t = 0; t < nt; ++t) {
      uint64_t a = set_components(base, (uint64_t)left[t], qubits, k);
      uint64_t b = set_components(base, (uint64_t)right[t], qubits, k);
      double tr = wf[2 * a], ti = wf[2 * a + 1];
      wf[2 * a] = wf[2 * b];
      wf[2 * a + 1] = wf[2 * b + 1];
      wf[2 * b] = tr;
      wf[2 * b + 1] = ti;
    }
  }
  free(left);
  free(right);
}

/* measurement.lisp:10-41 (force-measurement on a pure-state) */
void orc_force_measurement(double *wf, int nq, int measured_value, int q,
                           double excited_probability) {
  int annihilated = 1 - measured_value;
  double inv_norm = (annihilated == 0) ? 1.0 / sqrt(excited_probability)
                                       : 1.0 / sqrt(1.0 - excited_probability);
  uint64_t len = 1ull << nq;
  int par = nq >= g_threshold && g_workers > 1;
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t i = 0; i < (int64_t)len; ++i) {
    if ((int)(((uint64_t)i >> q) & 1ull) == annihilated) {
      wf[2 * i] = 0.0;
      wf[2 * i + 1] = 0.0;
    } else {
      wf[2 * i] = inv_norm * wf[2 * i];
      wf[2 * i + 1] = inv_norm * wf[2 * i + 1];
    }
  }
}

/* measurement.lisp:87-105 (measure) */
int orc_measure(double *wf, int nq, int q, double draw, int *draw_used,
                double *p1_out) {
  double p1 = orc_excited_probability(wf, nq, q);
  int bit;
  if (p1 == 0.0) {
    bit = 0;
    if (draw_used) *draw_used = 0;
  } else {
    bit = (draw <= p1) ? 1 : 0;
    if (draw_used) *draw_used = 1;
  }
  orc_force_measurement(wf, nq, bit, q, p1);
  if (p1_out) *p1_out = p1;
  return bit;
}

/* compile-gate.lisp:221-254 (generate-single-qubit-measurement-code) */
int orc_measure_compiled(double *wf, int nq, int q, double draw,
                         double *p0_out) {
  double p0 = orc_ground_probability(wf, nq, q);
  int keep_zero = draw < p0;
  int keep_bit = keep_zero ? 0 : 1;
  double inv_norm = keep_zero ? 1.0 / sqrt(p0) : 1.0 / sqrt(1.0 - p0);
  uint64_t len = 1ull << nq;
  int par = len > (1ull << g_threshold) && g_workers > 1; /* pdotimes */
#pragma omp parallel for if (par) num_threads(g_workers) schedule(static)
  for (int64_t i = 0; i < (int64_t)len; ++i) {
    int abit = (int)(((uint64_t)i >> q) & 1ull);
    double f = inv_norm * (double)(abit == keep_bit);
    wf[2 * i] = f * wf[2 * i];
    wf[2 * i + 1] = f * wf[2 * i + 1];
  }
  if (p0_out) *p0_out = p0;
  return keep_bit;
}

/* measurement.lisp:179-225: smallest b with C(b) > p by bisection, where the
 * lower-half sums are psum-dotimes over [min, mid). */
uint64_t orc_sample_bisect(const double *wf, uint64_t len, double p) {
  uint64_t min = 0, max = len;
  double sum_lt = 0.0;
  while (min != max - 1) {
    uint64_t mid = min + (max - min) / 2; /* midpoint, :172-177 */
    sum_body b = {wf, min, 0, 0};
    double sum = sum_lt + psum_dotimes(&b, mid - min);
    if (sum <= p) {
      min = mid;
      sum_lt = sum;
    } else {
      max = mid;
    }
  }
  return min;
}

/* measurement.lisp:128-143 (measure-all-state on a pure-state) */
uint64_t orc_measure_all(double *wf, int nq, double draw) {
  uint64_t len = 1ull << nq;
  uint64_t b = orc_sample_bisect(wf, len, draw);
  orc_bring_to_zero(wf, len);
  /* rotatef amp[0] <-> amp[b] */
  double tr = wf[0], ti = wf[1];
  wf[0] = wf[2 * b];
  wf[1] = wf[2 * b + 1];
  wf[2 * b] = tr;
  wf[2 * b + 1] = ti;
  return b;
}

/* wavefunction.lisp:382-395 (cumulative-distribution-function) */
void orc_cdf(const double *wf, uint64_t len, double *cdf) {
  double s = 0.0;
  for (uint64_t i = 0; i < len; ++i) {
    s += prob(wf, i);
    cdf[i] = s;
  }
}

/* measurement.lisp:246-288 (sample-wavefunction-multiple-times), the draws
 * supplied by the caller instead of (random 1.0d0). */
void orc_sample_multiple(const double *wf, uint64_t len, const double *draws,
                         uint64_t nshots, uint64_t *out) {
  double *cdf = (double *)malloc(sizeof(double) * (len ? len : 1));
  orc_cdf(wf, len, cdf);
  for (uint64_t t = 0; t < nshots; ++t) {
    double p = draws[t];
    uint64_t min = 0, max = len - 1;
    for (;;) {
      uint64_t mid = min + (max - min) / 2;
      if (min == max) { out[t] = min; break; }
      if (max - min == 1) { out[t] = (cdf[min] < p) ? max : min; break; }
      if (cdf[mid] < p) min = mid; else max = mid;
    }
  }
  free(cdf);
}

/* app/src/api/expectation.lisp:80-84 (inner-product) */
void orc_inner(const double *a, const double *b, uint64_t len, double *re,
               double *im) {
  double sr = 0.0, si = 0.0;
  for (uint64_t i = 0; i < len; ++i) {
    double ar = a[2 * i], ai = -a[2 * i + 1];
    double br = b[2 * i], bi = b[2 * i + 1];
    sr = sr + (ar * br - ai * bi);
    si = si + (ar * bi + ai * br);
  }
  *re = sr;
  *im = si;
}

/* ---- quil/stdgates.quil gate matrices ---------------------------------- */

static void setc(double *m, int dim, int r, int c, double re, double im) {
  m[2 * (r * dim + c)] = re;
  m[2 * (r * dim + c) + 1] = im;
}

static void eye(double *m, int dim) {
  memset(m, 0, sizeof(double) * 2 * dim * dim);
  for (int i = 0; i < dim; ++i) setc(m, dim, i, i, 1.0, 0.0);
}

int orc_gate_matrix(const char *name, const double *params, int nparams,
                    double *m, int *k) {
#define NEED(n) do { if (nparams != (n)) return -1; } while (0)
  const double r2 = 1.0 / sqrt(2.0);
  if (!strcmp(name, "I")) { NEED(0); *k = 1; eye(m, 2); return 0; }
  if (!strcmp(name, "X")) {
    NEED(0); *k = 1; memset(m, 0, sizeof(double) * 8);
    setc(m, 2, 0, 1, 1, 0); setc(m, 2, 1, 0, 1, 0); return 0;
  }
  if (!strcmp(name, "Y")) {
    NEED(0); *k = 1; memset(m, 0, sizeof(double) * 8);
    setc(m, 2, 0, 1, 0, -1); setc(m, 2, 1, 0, 0, 1); return 0;
  }
  if (!strcmp(name, "Z")) {
    NEED(0); *k = 1; eye(m, 2); setc(m, 2, 1, 1, -1, 0); return 0;
  }
  if (!strcmp(name, "H")) {
    NEED(0); *k = 1;
    setc(m, 2, 0, 0, r2, 0); setc(m, 2, 0, 1, r2, 0);
    setc(m, 2, 1, 0, r2, 0); setc(m, 2, 1, 1, -r2, 0); return 0;
  }
  if (!strcmp(name, "RX")) {
    NEED(1); *k = 1; double c = cos(params[0] / 2), s = sin(params[0] / 2);
    setc(m, 2, 0, 0, c, 0); setc(m, 2, 0, 1, 0, -s);
    setc(m, 2, 1, 0, 0, -s); setc(m, 2, 1, 1, c, 0); return 0;
  }
  if (!strcmp(name, "RY")) {
    NEED(1); *k = 1; double c = cos(params[0] / 2), s = sin(params[0] / 2);
    setc(m, 2, 0, 0, c, 0); setc(m, 2, 0, 1, -s, 0);
    setc(m, 2, 1, 0, s, 0); setc(m, 2, 1, 1, c, 0); return 0;
  }
  if (!strcmp(name, "RZ")) {
    NEED(1); *k = 1; double h = params[0] / 2; memset(m, 0, sizeof(double) * 8);
    setc(m, 2, 0, 0, cos(-h), sin(-h)); setc(m, 2, 1, 1, cos(h), sin(h));
    return 0;
  }
  if (!strcmp(name, "S")) { NEED(0); *k = 1; eye(m, 2); setc(m, 2, 1, 1, 0, 1); return 0; }
  if (!strcmp(name, "T")) {
    NEED(0); *k = 1; eye(m, 2);
    setc(m, 2, 1, 1, cos(M_PI / 4), sin(M_PI / 4)); return 0;
  }
  if (!strcmp(name, "PHASE")) {
    NEED(1); *k = 1; eye(m, 2);
    setc(m, 2, 1, 1, cos(params[0]), sin(params[0])); return 0;
  }
  if (!strcmp(name, "CNOT")) {
    NEED(0); *k = 2; memset(m, 0, sizeof(double) * 32);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 1, 1, 0);
    setc(m, 4, 2, 3, 1, 0); setc(m, 4, 3, 2, 1, 0); return 0;
  }
  if (!strcmp(name, "CZ")) { NEED(0); *k = 2; eye(m, 4); setc(m, 4, 3, 3, -1, 0); return 0; }
  if (!strcmp(name, "CPHASE") || !strcmp(name, "CPHASE00") ||
      !strcmp(name, "CPHASE01") || !strcmp(name, "CPHASE10")) {
    NEED(1); *k = 2; eye(m, 4);
    int slot = !strcmp(name, "CPHASE") ? 3 : !strcmp(name, "CPHASE00") ? 0
             : !strcmp(name, "CPHASE01") ? 1 : 2;
    setc(m, 4, slot, slot, cos(params[0]), sin(params[0])); return 0;
  }
  if (!strcmp(name, "SWAP")) {
    NEED(0); *k = 2; memset(m, 0, sizeof(double) * 32);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 2, 1, 0);
    setc(m, 4, 2, 1, 1, 0); setc(m, 4, 3, 3, 1, 0); return 0;
  }
  if (!strcmp(name, "ISWAP")) {
    NEED(0); *k = 2; memset(m, 0, sizeof(double) * 32);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 2, 0, 1);
    setc(m, 4, 2, 1, 0, 1); setc(m, 4, 3, 3, 1, 0); return 0;
  }
  if (!strcmp(name, "SQISWAP")) {
    NEED(0); *k = 2; memset(m, 0, sizeof(double) * 32);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 1, r2, 0); setc(m, 4, 1, 2, 0, r2);
    setc(m, 4, 2, 1, 0, r2); setc(m, 4, 2, 2, r2, 0); setc(m, 4, 3, 3, 1, 0);
    return 0;
  }
  if (!strcmp(name, "PSWAP")) {
    NEED(1); *k = 2; memset(m, 0, sizeof(double) * 32);
    double c = cos(params[0]), s = sin(params[0]);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 2, c, s);
    setc(m, 4, 2, 1, c, s); setc(m, 4, 3, 3, 1, 0); return 0;
  }
  if (!strcmp(name, "RZZ")) {
    NEED(1); *k = 2; memset(m, 0, sizeof(double) * 32);
    double h = params[0] / 2;
    setc(m, 4, 0, 0, cos(-h), sin(-h)); setc(m, 4, 1, 1, cos(h), sin(h));
    setc(m, 4, 2, 2, cos(h), sin(h)); setc(m, 4, 3, 3, cos(-h), sin(-h));
    return 0;
  }
  if (!strcmp(name, "RXX") || !strcmp(name, "RYY")) {
    NEED(1); *k = 2; memset(m, 0, sizeof(double) * 32);
    double c = cos(params[0] / 2), s = sin(params[0] / 2);
    double corner = !strcmp(name, "RXX") ? -s : s;
    for (int i = 0; i < 4; ++i) setc(m, 4, i, i, c, 0);
    setc(m, 4, 0, 3, 0, corner); setc(m, 4, 3, 0, 0, corner);
    setc(m, 4, 1, 2, 0, -s); setc(m, 4, 2, 1, 0, -s); return 0;
  }
  if (!strcmp(name, "PISWAP") || !strcmp(name, "XY")) {
    NEED(1); *k = 2; memset(m, 0, sizeof(double) * 32);
    double c = cos(params[0] / 2), s = sin(params[0] / 2);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 1, c, 0); setc(m, 4, 1, 2, 0, s);
    setc(m, 4, 2, 1, 0, s); setc(m, 4, 2, 2, c, 0); setc(m, 4, 3, 3, 1, 0);
    return 0;
  }
  if (!strcmp(name, "FSIM")) {
    NEED(2); *k = 2; memset(m, 0, sizeof(double) * 32);
    double c = cos(params[0] / 2), s = sin(params[0] / 2);
    setc(m, 4, 0, 0, 1, 0); setc(m, 4, 1, 1, c, 0); setc(m, 4, 1, 2, 0, s);
    setc(m, 4, 2, 1, 0, s); setc(m, 4, 2, 2, c, 0);
    setc(m, 4, 3, 3, cos(params[1]), sin(params[1])); return 0;
  }
  if (!strcmp(name, "CCNOT")) {
    NEED(0); *k = 3; eye(m, 8);
    setc(m, 8, 6, 6, 0, 0); setc(m, 8, 7, 7, 0, 0);
    setc(m, 8, 6, 7, 1, 0); setc(m, 8, 7, 6, 1, 0); return 0;
  }
  if (!strcmp(name, "CSWAP")) {
    NEED(0); *k = 3; eye(m, 8);
    setc(m, 8, 5, 5, 0, 0); setc(m, 8, 6, 6, 0, 0);
    setc(m, 8, 5, 6, 1, 0); setc(m, 8, 6, 5, 1, 0); return 0;
  }
  return -1;
#undef NEED
}
