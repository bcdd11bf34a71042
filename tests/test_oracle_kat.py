"""Pin the CPU oracle to the reference's own known-answer tests.

Every case comes from tests/golden/reference_kats.json, which transcribes
the reference QVM's test suite (each entry cites its file:line).
"""
import json
import os

import numpy as np
import pytest

from qvm_gb300 import circuits, gates

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def kat_vector(probs_single):
    """(make-vector n (sqrt x) ...) with x a single-float: sqrt in single
    precision, then coerced to complex double."""
    return np.sqrt(np.array(probs_single, dtype=np.float32)).astype(np.complex128)


def lisp_accumulated_draws(step, count):
    """(loop for p from 0.0d0 by step) -- repeated double additions."""
    out, p = [], 0.0
    for _ in range(count):
        out.append(p)
        p = p + step
    return out


def test_inject_eject_bit(oracle):
    k = KATS["inject_bit"]
    for n, want in k["cases"]:
        assert oracle.inject_bit(k["source"], n) == want
    k = KATS["eject_bit"]
    for x, n in k["cases"]:
        assert oracle.eject_bit(x, n) == k["target"]


def test_index_to_address(oracle):
    k = KATS["index_to_address"]
    for q, want in enumerate(k["addresses"]):
        assert oracle.index_to_address(k["index"], q, k["state"]) == want


def test_subdivide(oracle):
    k = KATS["subdivide"]
    for c in k["cases"]:
        assert [list(r) for r in oracle.subdivide(c["total"], k["workers"])] == c["ranges"]


def test_nat_tuple_order():
    k = KATS["nat_tuple"]
    # circuits.app converts Quil argument order to nat-tuple order
    assert circuits.app("CCNOT", (), *k["args"])[1] == k["tuple"]


def test_qft2_table(oracle):
    k = KATS["qft2"]
    for prep, expected in zip(k["preparations"], k["expected"]):
        wf = oracle.zero_state(2)
        for q in prep:
            oracle.apply_matrix_operator(wf, oracle.gate_matrix("X"), [q])
        for m, qs in circuits.qft_examples_order([0, 1]):
            oracle.apply_matrix_operator(wf, m, qs)
        exp = np.array([complex(a, b) for a, b in expected])
        assert np.all(np.abs(wf.real - exp.real) < k["tolerance"])
        assert np.all(np.abs(wf.imag - exp.imag) < k["tolerance"])


def test_sample_wavefunction_bisection(oracle):
    for c in KATS["sample_wavefunction"]["cases"]:
        v = kat_vector(c["probs_single"])
        draws = c["draws"]
        if isinstance(draws, str):
            draws = lisp_accumulated_draws(0.1, len(c["expected"]))
        got = [oracle.sample_bisect(v, p) for p in draws]
        assert got == c["expected"], (c, got)


def test_cdf(oracle):
    k = KATS["cdf"]
    for c in k["cases"]:
        if "sqrt_single" in c:
            v = kat_vector(c["sqrt_single"])
        else:
            v = np.array(c["amps"], dtype=np.complex128)
        if len(v) == 0:
            assert len(c["cdf"]) == 0
            continue
        got = oracle.cdf(np.ascontiguousarray(v))
        np.testing.assert_allclose(got, c["cdf"], rtol=k["rel_tol"])


def test_measure_all_basis_states(oracle):
    n = KATS["measure_all_basis"]["n"]
    for i in range(1 << n):
        wf = oracle.zero_state(n)
        for q in range(n):
            if (i >> q) & 1:
                oracle.apply_matrix_operator(wf, oracle.gate_matrix("X"), [q])
        b = oracle.measure_all(wf, 0.5)
        assert b == i
        assert wf[i] == 1.0 and np.count_nonzero(wf) == 1


def test_gate_tables_agree(oracle):
    """The host gate table (quil/stdgates.quil restated in Python) matches
    the oracle's restatement in C."""
    rng = np.random.default_rng(0)
    for name, (npar, _) in gates.STANDARD_GATES.items():
        params = rng.uniform(-3, 3, npar)
        try:
            om = oracle.gate_matrix(name, *params)
        except KeyError:
            pytest.fail(f"oracle lacks {name}")
        np.testing.assert_allclose(gates.gate_matrix(name, *params), om, atol=1e-15)


def test_xy_equals_piswap(oracle):
    """tests/gate-tests.lisp:115-127"""
    for s in range(10):
        wf = circuits.random_state(2, seed=s)
        a, b = wf.copy(), wf.copy()
        oracle.apply_matrix_operator(a, oracle.gate_matrix("XY", np.pi / 2), [0, 1])
        oracle.apply_matrix_operator(b, oracle.gate_matrix("PISWAP", np.pi / 2), [0, 1])
        np.testing.assert_allclose(a, b, rtol=1e-5)


def test_bell_and_hadamard(oracle):
    """tests/gate-tests.lisp:13-26 and :75-89"""
    for n in range(1, 11):
        wf = oracle.zero_state(n)
        oracle.apply_matrix_operator(wf, oracle.gate_matrix("H"), [0])
        for i in range(1, n):
            oracle.apply_matrix_operator(wf, oracle.gate_matrix("CNOT"), [i, 0])
        p = np.abs(wf) ** 2
        assert abs(p[0] - 0.5) < 1e-4 and abs(p[-1] - 0.5) < 1e-4
        wf = oracle.zero_state(n)
        for q in range(n):
            oracle.apply_matrix_operator(wf, oracle.gate_matrix("H"), [q])
        assert np.all(np.abs(np.abs(wf) ** 2 - 2.0 ** -n) < 1e-4)


def test_permutation_transpositions(oracle):
    """tests/utilities-tests.lisp:39-49: applying the transpositions to the
    identity reproduces the permutation."""
    rng = np.random.default_rng(5)
    for _ in range(200):
        n = 2 ** int(rng.integers(1, 6))
        perm = list(rng.permutation(n))
        ident = list(range(n))
        for a, b in oracle.permutation_to_transpositions(perm):
            ident[a], ident[b] = ident[b], ident[a]
        assert ident == perm


def test_permutation_gate_matches_matrix(oracle):
    """Compiled permutation gates (rotatef transpositions) equal the matrix
    product with M[j, perm[j]] = 1."""
    rng = np.random.default_rng(6)
    for _ in range(20):
        k = int(rng.integers(1, 4))
        perm = rng.permutation(1 << k)
        qs = list(rng.choice(6, k, replace=False))
        wf = circuits.random_state(6, seed=int(rng.integers(1000)))
        a, b = wf.copy(), wf.copy()
        oracle.apply_permutation(a, perm, qs)
        oracle.apply_matrix_operator(b, gates.permutation_matrix(perm), qs)
        np.testing.assert_array_equal(a, b)


def test_measure_conventions(oracle):
    """measure (src/measurement.lisp:87-105) vs the compiled measurement
    (src/compile-gate.lisp:221-254) on a |+> qubit."""
    wf = oracle.zero_state(1)
    oracle.apply_matrix_operator(wf, oracle.gate_matrix("H"), [0])
    a = wf.copy()
    bit, used, p1 = oracle.measure(a, 0, 0.3)
    assert used and bit == 1 and abs(p1 - 0.5) < 1e-15
    assert abs(abs(a[1]) - 1) < 1e-15 and a[0] == 0
    b = wf.copy()
    bit, p0 = oracle.measure_compiled(b, 0, 0.3)
    assert bit == 0 and abs(b[0]) == pytest.approx(1.0)
    # p1 = 0: no draw consumed, bit 0
    z = oracle.zero_state(2)
    bit, used, p1 = oracle.measure(z, 1, 0.0)
    assert bit == 0 and not used and p1 == 0.0


def test_unit_norm_after_measurements(oracle):
    """tests/measurement-tests.lisp:88-97"""
    rng = np.random.default_rng(7)
    for n in range(5, 12):
        wf = oracle.zero_state(n)
        for q in range(n):
            oracle.apply_matrix_operator(wf, oracle.gate_matrix("H"), [q])
            oracle.measure(wf, q, rng.random())
        assert abs(oracle.norm(wf) - 1.0) < 1e-12


def test_qft_is_dft(oracle):
    """Property of the QFT workload: it maps a state to its discrete Fourier
    transform (up to the bit-reversal convention), checked with numpy."""
    n = 6
    wf = circuits.random_state(n, seed=11)
    ref = np.fft.ifft(wf) * np.sqrt(len(wf))
    out = wf.copy()
    for m, qs in circuits.qft(n):
        oracle.apply_matrix_operator(out, m, qs)
    ok = np.allclose(out, ref, atol=1e-12) or np.allclose(out, np.fft.fft(wf) / np.sqrt(len(wf)), atol=1e-12)
    assert ok


def test_parallel_sums_match_serial(oracle):
    """psum serial == parallel (tests/linear-algebra-tests.lisp:17-52) for the
    oracle's worker-parallel reductions."""
    wf = circuits.random_state(20, seed=3)
    oracle.set_workers(1)
    s1 = oracle.excited_probability(wf, 7)
    b1 = oracle.sample_bisect(wf, 0.37)
    oracle.set_workers(4, threshold=10)
    s4 = oracle.excited_probability(wf, 7)
    b4 = oracle.sample_bisect(wf, 0.37)
    oracle.set_workers(1, threshold=19)
    assert abs(s1 - s4) < 1e-13
    assert b1 == b4
