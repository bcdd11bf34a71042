"""GPU: batches of small, uneven programs in one persistent launch.

Each program's final state matches the oracle (1e-12 per amplitude in FP64,
2e-6 in FP32), its shots are the oracle's CDF samples on the same draws
(except draws within 1e-12 of a boundary; FP32 samples the renormalised
distribution), and a program's results are identical alone and inside a
mixed batch."""
import numpy as np
import pytest

from qvm_gb300 import circuits, gates
from qvm_gb300.batch import ProgramBatch

pytestmark = pytest.mark.gpu


def _programs(rng, nmax, count):
    progs = []
    for i in range(count):
        n = int(rng.integers(1, nmax + 1))
        fam = i % 3
        if fam == 0 and n >= 2:
            gs = circuits.random_su_circuit(n, depth=3, seed=int(rng.integers(1 << 20)))
        elif fam == 1:
            gs = circuits.random_layers(n, layers=2, seed=int(rng.integers(1 << 20))) if n >= 2 \
                else [(gates.gate_matrix("H"), [0])]
        else:
            gs = [(gates.gate_matrix("H"), [q]) for q in range(n)]
            if n >= 3:  # a 3-qubit block (Toffoli) and a 3-qubit Haar block
                gs.append((gates.gate_matrix("CCNOT"), [0, 1, 2]))
                gs.append((gates.haar_special_unitary(rng, 8), [n - 1, 0, n // 2]))
        progs.append((n, gs, int(rng.integers(0, 300))))
    return progs


def _oracle_state(oracle, n, gs):
    wf = oracle.zero_state(n)
    for m, qs in gs:
        oracle.apply_matrix_operator(wf, m, qs)
    return wf


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_small_batch_matches_oracle(gpu, oracle, prec):
    rng = np.random.default_rng(3 if prec == "fp64" else 4)
    nmax = 12 if prec == "fp64" else 13
    progs = _programs(rng, nmax, 40) + [(nmax, circuits.random_su_circuit(nmax, 4, seed=9), 1000)]
    draws = [rng.random(k) for _, _, k in progs]
    b = ProgramBatch(progs, prec)
    shots = b.run(draws)
    tol = 1e-12 if prec == "fp64" else 2e-6
    for i, (n, gs, k) in enumerate(progs):
        want = _oracle_state(oracle, n, gs)
        got = b.state(i)
        assert np.max(np.abs(got - want)) < tol, (i, n, prec)
        ref = want if prec == "fp64" else got.astype(np.complex64).astype(np.complex128)
        tot = 1.0 if prec == "fp64" else float(np.sum(np.abs(ref) ** 2))
        if k:
            wsh = oracle.sample_multiple(ref, draws[i] * tot)
            cdf = np.cumsum(np.abs(ref) ** 2)
            near = np.array([np.min(np.abs(cdf - d * tot)) < 1e-12 for d in draws[i]])
            assert ((shots[i] == wsh) | near).all(), (i, n, prec)
    b.free()


def test_small_batch_alone_equals_in_mix(gpu):
    rng = np.random.default_rng(5)
    progs = _programs(rng, 13, 30)
    draws = [rng.random(k) for _, _, k in progs]
    mix = ProgramBatch(progs, "fp32")
    mix_shots = mix.run(draws)
    mix_shots2 = mix.run(draws)  # replay of the captured graph
    for i in (0, 7, 29):
        alone = ProgramBatch([progs[i]], "fp32")
        s = alone.run([draws[i]])
        np.testing.assert_array_equal(alone.state(0), mix.state(i))
        np.testing.assert_array_equal(s[0], mix_shots[i])
        np.testing.assert_array_equal(mix_shots2[i], mix_shots[i])
        alone.free()
    mix.free()


def test_small_batch_rejects_bad_programs(gpu):
    from qvm_gb300 import QVMGError
    with pytest.raises(QVMGError, match="qubits outside"):
        ProgramBatch([(13, [], 0)], "fp64")
    with pytest.raises(QVMGError, match="out of range"):
        ProgramBatch([(3, [(np.eye(2), [3])], 0)], "fp32")
    b = ProgramBatch([(2, [(np.eye(4), [0, 1])], 2)], "fp32")
    with pytest.raises(QVMGError, match=r"\[0, 1\]"):
        b.run([np.array([0.5, 1.5])])
    b.free()
