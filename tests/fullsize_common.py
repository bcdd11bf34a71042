"""Fingerprints of full-size wavefunctions (test infrastructure).

A 28- or 30-qubit state is 4-16 GiB, too large to commit.  Its fingerprint
is small and still pins every amplitude's position and value:

- the amplitudes at ~4200 fixed indices (uniform random ones plus every
  single-bit and all-but-one-bit index), compared at 1e-12 each;
- 2048 weighted block sums S_b = sum_i a_i * w(i) over contiguous blocks,
  with w(i) in [-0.5, 0.5) an integer hash of the index (exact in FP64,
  the same on every machine).  A misplaced or wrong amplitude anywhere moves
  its block's sum by |a| * |w|, orders of magnitude above the tolerance.

The same functions make the committed fixtures (``golden/make_fullsize.py``)
and check the device's states in ``test_gpu_fullsize_oracle.py``.
"""
from __future__ import annotations

import numpy as np

FP_BLOCKS = 2048
FP_SAMPLES = 4096
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def fingerprint_indices(n: int, seed: int = 12345) -> np.ndarray:
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, 1 << n, FP_SAMPLES, dtype=np.uint64)
    full = (1 << n) - 1
    special = [0, full] + [1 << q for q in range(n)] + [full ^ (1 << q) for q in range(n)]
    return np.unique(np.concatenate([idx, np.array(special, dtype=np.uint64)]))


def index_weights(i0: int, count: int) -> np.ndarray:
    i = np.arange(i0, i0 + count, dtype=np.uint64)
    h = i * _GOLD  # wraps modulo 2^64
    h ^= h >> np.uint64(29)
    h = h * _GOLD
    return (h >> np.uint64(40)).astype(np.float64) / float(1 << 24) - 0.5


def block_sums(wf: np.ndarray) -> np.ndarray:
    n_amp = len(wf)
    blk = n_amp // FP_BLOCKS
    out = np.empty(FP_BLOCKS, dtype=np.complex128)
    for b in range(FP_BLOCKS):
        seg = wf[b * blk:(b + 1) * blk]
        w = index_weights(b * blk, blk)
        out[b] = complex(np.dot(np.ascontiguousarray(seg.real), w),
                         np.dot(np.ascontiguousarray(seg.imag), w))
    return out


def fingerprint(wf: np.ndarray, n: int) -> dict:
    idx = fingerprint_indices(n)
    return {"idx": idx, "amps": wf[idx.astype(np.int64)].copy(), "block_sums": block_sums(wf)}


def compare(got: np.ndarray, n: int, fx, amp_tol: float = 1e-12, sum_tol: float = 1e-12):
    """Largest amplitude and block-sum deviations of ``got`` from the fixture."""
    idx = np.asarray(fx["idx"], dtype=np.uint64)
    assert (idx == fingerprint_indices(n)).all(), "fingerprint indices changed"
    amp_err = float(np.max(np.abs(got[idx.astype(np.int64)] - fx["amps"])))
    sum_err = float(np.max(np.abs(block_sums(got) - fx["block_sums"])))
    return amp_err, sum_err


def cdf_boundary_exemptions(wf: np.ndarray, draws: np.ndarray, shots: np.ndarray,
                            serial_cdf: np.ndarray, tau: float = 1e-12) -> np.ndarray:
    """Draws whose sample may legitimately differ between two CDF evaluations.

    The reference's CDF (src/wavefunction.lisp:382-395) is a serial FP64
    prefix sum; over 2^30 terms its own rounding reaches ~1e-12, so the
    1e-12 boundary rule is widened by that measured rounding.  For each draw
    d with oracle sample i the bracketing boundaries C(i-1) < d <= C(i) are
    recomputed in extended precision (pairwise block sums, then long-double
    prefix sums); the draw is exempt when it lies within
    tau + |serial - extended| of either boundary.
    """
    probs_chunk = 1 << 22
    n_amp = len(wf)
    nchunks = max(1, n_amp // probs_chunk)
    chunk = n_amp // nchunks
    # extended-precision chunk totals
    tot = np.zeros(nchunks, dtype=np.longdouble)
    for c in range(nchunks):
        seg = wf[c * chunk:(c + 1) * chunk]
        p = seg.real * seg.real + seg.imag * seg.imag
        tot[c] = np.sum(p.astype(np.longdouble))
    base = np.concatenate([[np.longdouble(0)], np.cumsum(tot)])
    need = np.unique(np.concatenate([shots.astype(np.int64), np.maximum(shots.astype(np.int64) - 1, 0)]))
    exact = {}
    for c in np.unique(need // chunk):
        seg = wf[c * chunk:(c + 1) * chunk]
        p = (seg.real * seg.real + seg.imag * seg.imag).astype(np.longdouble)
        cs = base[c] + np.cumsum(p)
        for j in need[(need // chunk) == c]:
            exact[int(j)] = cs[j - c * chunk]
    exempt = np.zeros(len(draws), dtype=bool)
    for t, (d, i) in enumerate(zip(draws, shots.astype(np.int64))):
        hi_e = exact[int(i)]
        lo_e = exact[int(i) - 1] if i > 0 else np.longdouble(0)
        hi_s = serial_cdf[i]
        lo_s = serial_cdf[i - 1] if i > 0 else 0.0
        widen = max(abs(float(hi_s - hi_e)), abs(float(lo_s - lo_e)))
        margin = tau + widen
        d_l = np.longdouble(d)
        if (d_l - lo_e) < margin or (hi_e - d_l) < margin:
            exempt[t] = True
    return exempt
