"""GPU parity of the noisy pure-state paths against the oracle.

- the reduced density matrix against numpy;
- the stochastic Kraus step against the reference's algorithm restated on
  the oracle (copy, apply K_j, add its norm, stop once the sum reaches the
  draw, normalise), for the same draws;
- the reference's noisy-qvm and depolarizing-qvm tests
  (tests/noisy-qvm-tests.lisp): every expected outcome shows up.
"""
import random

import numpy as np
import pytest

from qvm_gb300 import CudaPureState, circuits, gates
from qvm_gb300.noisy import (DepolarizingQVM, NoisyQVM, make_pauli_noise_map,
                             make_pauli_perturbed_1q_gate)

pytestmark = pytest.mark.gpu


def upload(wf, prec="fp64"):
    n = int(np.log2(len(wf)))
    s = CudaPureState(n, prec)
    s.set_state_elements(wf)
    return s


def numpy_rdm(wf, qubits):
    n = int(np.log2(len(wf)))
    k = len(qubits)
    idx = np.arange(len(wf))
    sub = np.zeros(len(wf), dtype=np.int64)
    for j, q in enumerate(qubits):
        sub |= ((idx >> q) & 1) << j
    rest = idx.copy()
    for q in sorted(qubits, reverse=True):
        rest = ((rest >> (q + 1)) << q) | (rest & ((1 << q) - 1))
    m = np.zeros((1 << (n - k), 1 << k), dtype=np.complex128)
    m[rest, sub] = wf
    return m.T @ m.conj()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_reduced_density_matrix(gpu, prec):
    rng = np.random.default_rng(2)
    for n in (1, 2, 5, 12, 20):
        wf = circuits.random_state(n, seed=n)
        s = upload(wf, prec)
        ref = s.state_elements()
        for k in (1, 2):
            if k > n:
                continue
            for _ in range(4):
                qs = [int(x) for x in rng.permutation(n)[:k]]
                got = s.reduced_density_matrix(qs)
                np.testing.assert_allclose(got, numpy_rdm(ref, qs), atol=1e-13)
                np.testing.assert_array_equal(got, s.reduced_density_matrix(qs))
        s.free()


def oracle_kraus(oracle, wf, ops, qubits, r):
    summed = 0.0
    for j, k in enumerate(ops):
        trial = oracle.apply_matrix_operator(wf.copy(), k, qubits)
        summed += float(np.sum(np.abs(trial) ** 2))
        if summed >= r:
            break
    return j, trial / np.linalg.norm(trial)


def random_kraus_map(rng, k, nops):
    """Kraus operators from the blocks of a random isometry."""
    d = 1 << k
    v = gates.haar_unitary(rng, d * nops)[:, :d]
    return [v[j * d:(j + 1) * d, :] for j in range(nops)]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_apply_kraus_matches_reference_algorithm(gpu, oracle, prec):
    rng = np.random.default_rng(4)
    n = 11
    tol = 1e-12 if prec == "fp64" else 3e-6
    for trial in range(24):
        k = 1 + trial % 2
        nops = [1, 2, 3, 4, 6][trial % 5]
        ops = random_kraus_map(rng, k, nops)
        qs = [int(x) for x in rng.permutation(n)[:k]]
        wf = circuits.random_state(n, seed=trial)
        s = upload(wf, prec)
        wf = s.state_elements()
        r = float(rng.random())
        j, p = s.apply_kraus(ops, qs, r)
        wj, want = oracle_kraus(oracle, wf, ops, qs, r)
        assert j == wj
        np.testing.assert_allclose(s.state_elements(), want, atol=tol)
        s.free()


def test_pauli_noise_maps():
    ops = make_pauli_noise_map(0.1, 0.2, 0.3)
    assert len(ops) == 4 and np.allclose(ops[0], np.sqrt(0.4) * np.eye(2))
    assert len(make_pauli_noise_map(1 / 3, 1 / 3, 1 / 3)) == 3
    acc = sum(k.conj().T @ k for k in make_pauli_perturbed_1q_gate("X", 0.25, 0.25, 0.25))
    assert np.allclose(acc, np.eye(2))


def _seen_all(results_desired, make_psi, tries=500):
    want = [np.asarray(v, dtype=np.complex128) for v in results_desired]
    while want and tries:
        tries -= 1
        psi = make_psi()
        want = [w for w in want if not np.allclose(w, psi, atol=1e-15, rtol=0)]
    return tries > 0


def test_noisy_x_gate(gpu):
    """test-noisy-x-gate (tests/noisy-qvm-tests.lisp:89-112)."""
    qvm = NoisyQVM(2, seed=1)
    qvm.load_program("X 0\nX 1")

    def run():
        qvm.reset_quantum_state()
        qvm.set_noisy_gate("X", [0], make_pauli_perturbed_1q_gate("X", 0.25, 0.25, 0.25))
        return qvm.run().amplitudes

    assert _seen_all([[0, 0, 0, 1], [0, 0, 1, 0], [0, 0, -1j, 0]], run)
    qvm.free()


def test_noisy_readout_and_measure_all(gpu):
    """test-noisy-readout-2q-qvm and test-noisy-measure-all
    (tests/noisy-qvm-tests.lisp:114-176)."""
    qvm = NoisyQVM(2, seed=2)
    qvm.load_program("DECLARE ro BIT[2]\nMEASURE 0 ro[0]\nMEASURE 1 ro[1]")
    seen, tries = {0, 1}, 500
    while seen and tries:
        tries -= 1
        qvm.reset_quantum_state()
        qvm.set_readout_povm(1, (0.8, 0.1, 0.2, 0.9))
        qvm.run()
        assert qvm.memory_ref("ro", 0) == 0
        seen.discard(qvm.memory_ref("ro", 1))
    assert tries > 0
    qvm.free()
    qvm = NoisyQVM(2, seed=3)
    qvm.load_program("X 0\nX 1")
    seen, tries = {(1, 1), (1, 0)}, 500
    while seen and tries:
        tries -= 1
        qvm.reset_quantum_state()
        qvm.set_readout_povm(1, (0.8, 0.1, 0.2, 0.9))
        qvm.run()
        seen.discard(tuple(qvm.measure_all()[1]))
    assert tries > 0
    qvm.free()


def test_depolarizing_qvm(gpu):
    """test-empty-program-depolarizing-qvm, test-simple-gate-noise and
    test-simple-measurement-noise (tests/noisy-qvm-tests.lisp:15-70)."""
    q = DepolarizingQVM(1, x=1 / 3, y=1 / 3, z=1 / 3, seed=4)
    q.load_program("")
    q.run()
    assert q.state.excited_probability(0) == 0.0
    q.load_program("X 0")

    def run():
        q.reset_quantum_state()
        return q.run().amplitudes

    assert _seen_all([[0, -1], [1, 0], [-1j, 0]], run)
    q.free()
    q = DepolarizingQVM(1, measure_x=1 / 5, seed=5)
    q.load_program("DECLARE ro BIT\nMEASURE 0 ro[0]")
    seen, tries = {0, 1}, 500
    while seen and tries:
        tries -= 1
        q.reset_quantum_state()
        q.reset_classical_memory()
        q.run()
        seen.discard(q.memory_ref("ro", 0))
    assert tries > 0
    q.free()


def test_depolarizing_trajectory_matches_oracle(gpu, oracle):
    """One seeded trajectory of a noisy circuit, replayed on the oracle with
    the same draws in the reference's order."""
    prog = "H 0\nCNOT 0 1\nRX(0.4) 2\nCZ 1 2\nH 2"
    from qvm_gb300 import quil as Q
    apps = Q.parse(prog).instructions
    for seed in range(6):
        q = DepolarizingQVM(3, x=0.2, y=0.15, z=0.1, seed=seed)
        q.load_program(prog)
        q.run()
        got = q.amplitudes
        q.free()
        rng = random.Random(seed)
        wf = oracle.zero_state(3)
        for a in apps:
            oracle.apply_matrix_operator(wf, a.matrix, a.qubits)
            for qb in a.args:
                if rng.random() < 0.45:
                    r = rng.random()
                    px, py = 0.2 / 0.45, 0.15 / 0.45
                    name = "X" if r < px else ("Y" if r - px < py else "Z")
                    oracle.apply_matrix_operator(wf, gates.gate_matrix(name), [qb])
        np.testing.assert_allclose(got, wf, atol=1e-14)
