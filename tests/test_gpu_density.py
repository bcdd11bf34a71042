"""GPU parity of the density-matrix QVM: rho after gate, noisy-gate and
measurement programs against numpy density matrices built from the oracle,
and the reference's density-qvm tests (tests/density-qvm-tests.lisp)."""
import random

import numpy as np
import pytest

from qvm_gb300 import gates
from qvm_gb300 import quil as Q
from qvm_gb300.density import DensityQVM, make_density_qvm
from qvm_gb300.noisy import make_pauli_perturbed_1q_gate

pytestmark = pytest.mark.gpu


def embed(m, nat_qubits, n):
    dim = 1 << n
    full = np.zeros((dim, dim), dtype=np.complex128)
    for col in range(dim):
        c = sum(((col >> q) & 1) << j for j, q in enumerate(nat_qubits))
        for r in range(1 << len(nat_qubits)):
            row = col
            for j, q in enumerate(nat_qubits):
                row = (row & ~(1 << q)) | (((r >> j) & 1) << q)
            full[row, col] += m[r, c]
    return full


def trace(q):
    return float(np.sum(q.probabilities()))


def purity(q):
    m = q.matrix_view()
    return float(np.trace(m @ m).real)


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_unitary_circuit(gpu, oracle, fused, prec):
    n = 6
    prog = "\n".join(f"RX({0.3 * (i + 1)}) {i}" for i in range(n)) + \
        "\nCNOT 0 1\nCNOT 2 3\nCZ 4 5\nH 3\nCPHASE(0.7) 5 1\nSWAP 0 4\nRY(1.2) 2"
    q = DensityQVM(n, precision=prec, fused=fused)
    q.load_program(prog).run()
    wf = oracle.zero_state(n)
    for a in Q.parse(prog).instructions:
        oracle.apply_matrix_operator(wf, a.matrix, a.qubits)
    tol = 1e-13 if prec == "fp64" else 2e-6
    np.testing.assert_allclose(q.matrix_view(), np.outer(wf, wf.conj()), atol=tol)
    assert abs(trace(q) - 1) < tol
    q.free()


@pytest.mark.parametrize("fused", [False, True])
def test_noisy_gates_fold_into_rho(gpu, fused):
    n = 4
    rng = np.random.default_rng(5)
    k2 = [np.sqrt(0.6) * gates.haar_unitary(rng, 4), np.sqrt(0.4) * gates.haar_unitary(rng, 4)]
    q = DensityQVM(n, fused=fused)
    q.set_noisy_gate("H", [1], make_pauli_perturbed_1q_gate("H", 0.1, 0.05, 0.2))
    q.set_noisy_gate("CNOT", [2, 0], k2)
    prog = "H 0\nH 1\nCNOT 2 0\nRX(0.4) 3\nCNOT 3 1\nH 1"
    q.load_program(prog).run()
    rho = np.zeros((16, 16), dtype=np.complex128)
    rho[0, 0] = 1
    for a in Q.parse(prog).instructions:
        key = (a.name, tuple(a.args))
        if key == ("H", (1,)):
            ops = make_pauli_perturbed_1q_gate("H", 0.1, 0.05, 0.2)
        elif key == ("CNOT", (2, 0)):
            ops = k2
        else:
            ops = [a.matrix]
        rho = sum(embed(k, a.qubits, n) @ rho @ embed(k, a.qubits, n).conj().T for k in ops)
    np.testing.assert_allclose(q.matrix_view(), rho, atol=1e-13)
    assert purity(q) < 1 - 1e-3
    q.free()


def test_reference_density_tests(gpu):
    # test-density-qvm-parametric-gate
    q = make_density_qvm(1)
    q.load_program("DEFGATE G(%a):\n    cos(%a), sin(%a)\n    -sin(%a), cos(%a)\nG(0.0) 0").run()
    assert abs(q.matrix_view()[0, 0].real - 1) < 1e-4
    q.free()
    # test-density-qvm-force-measurement-1q
    q = make_density_qvm(1)
    q.load_program("H 0").run()
    q.force_measurement(1, 0, 0.5)
    assert abs(trace(q) - 1) < 1e-14 and abs(q.matrix_view()[1, 1].real - 1) < 1e-14
    q.free()
    # test-density-qvm-force-measurement-4q
    q = make_density_qvm(4)
    q.load_program("H 0\nCNOT 0 1\nCNOT 1 3\nH 3").run()
    assert abs(trace(q) - 1) < 1e-14
    p = q.excited_probability(3)
    q.force_measurement(1, 3, p)
    assert abs(trace(q) - 1) < 1e-14
    q.free()
    # test-density-qvm-1q-purity / 2q-purity
    for p in (0.1, 0.4, 0.5, 0.6, 0.9):
        want = (1 - p) ** 2 + p ** 2
        q = make_density_qvm(1)
        q.set_density_matrix(np.diag([1 - p, p]))
        assert abs(purity(q) - want) < 1e-14
        q.load_program("H 0").run()
        assert abs(purity(q) - want) < 1e-14
        q.free()
        q = make_density_qvm(2)
        q.set_density_matrix(np.kron(np.diag([1 - p, p]), np.full((2, 2), 0.5)))
        assert abs(purity(q) - want) < 1e-14
        q.load_program("CNOT 0 1").run()
        assert abs(purity(q) - want) < 1e-14
        q.free()
    # test-density-qvm-1q-measure-discard
    q = make_density_qvm(1)
    q.load_program("H 0\nMEASURE 0").run()
    m = q.matrix_view()
    assert abs(m[0, 0].real - 0.5) < 1e-15 and abs(m[1, 1].real - 0.5) < 1e-15
    assert abs(m[0, 1]) == 0
    q.free()
    # test-density-qvm-noisy-x-gate
    q = DensityQVM(2)
    q.set_noisy_gate("X", [0], make_pauli_perturbed_1q_gate("X", 1.0, 0.0, 0.0))
    q.load_program("DECLARE ro BIT\nX 0\nMEASURE 0 ro").run()
    assert q.memory_ref("ro", 0) == 0
    q.free()


def test_density_readout_and_measure_all(gpu):
    """test-density-qvm-noisy-readout and test-density-qvm-noisy-measure-all."""
    q = DensityQVM(2, seed=7)
    q.load_program("DECLARE ro BIT[2]\nMEASURE 0 ro[0]\nMEASURE 1 ro[1]")
    seen, tries = {0, 1}, 500
    while seen and tries:
        tries -= 1
        q.reset_quantum_state()
        q.set_readout_povm(1, (0.8, 0.1, 0.2, 0.9))
        q.run()
        assert q.memory_ref("ro", 0) == 0
        seen.discard(q.memory_ref("ro", 1))
    assert tries > 0
    q.free()
    q = DensityQVM(2, seed=8)
    q.load_program("X 0\nX 1")
    seen, tries = {(1, 1), (1, 0)}, 500
    while seen and tries:
        tries -= 1
        q.reset_quantum_state()
        q.set_readout_povm(1, (0.8, 0.1, 0.2, 0.9))
        q.run()
        seen.discard(tuple(q.measure_all()[1]))
    assert tries > 0
    q.free()


def test_measure_matches_sequential_collapse(gpu):
    """Measurements and measure-all against a numpy density matrix collapsed
    with the same draws (src/measurement.lisp:43-105,145-150)."""
    n = 3
    prog = "H 0\nCNOT 0 1\nRY(0.9) 2\nCNOT 2 0"
    for seed in range(5):
        q = DensityQVM(n, seed=seed)
        q.set_noisy_gate("H", [0], make_pauli_perturbed_1q_gate("H", 0.1, 0.1, 0.1))
        q.load_program(prog).run()
        rho = q.matrix_view()
        rng = random.Random(seed)
        # the same sequence of measurements, qubit n-1 first, on the host
        _, bits = q.measure_all()
        idx = np.arange(1 << n)
        d = np.diag(rho).real.copy()
        mask = np.ones(1 << n, dtype=bool)
        want = [0] * n
        for qb in range(n - 1, -1, -1):
            p1 = d[mask & ((idx >> qb) & 1 == 1)].sum() / d[mask].sum()
            b = 0 if p1 == 0 else (1 if rng.random() <= p1 else 0)
            want[qb] = b
            mask &= ((idx >> qb) & 1) == b
        assert bits == want
        b = sum(v << i for i, v in enumerate(bits))
        m = q.matrix_view()
        assert m[b, b] == 1 and np.count_nonzero(m) == 1
        q.free()
