"""GPU parity of the server endpoints (qvm_gb300.api) and their C-ABI calls.

- marginal probabilities against numpy sums of the downloaded state;
- the multishot-measure trial replay against the oracle's per-trial
  measure on a fresh copy of the state, with the same draws (bit-exact,
  including the count of draws consumed);
- multishot's fast path against the trial-by-trial run of the same QVM;
- expectation values against the oracle;
- wire bytes against numpy's big-endian encoding.
"""
import random

import numpy as np
import pytest

from qvm_gb300 import CudaPureState, api, circuits, gates
from qvm_gb300 import quil as Q
from qvm_gb300.qvm import PureStateQVM

pytestmark = pytest.mark.gpu


def upload(wf, prec="fp64"):
    n = int(np.log2(len(wf)))
    s = CudaPureState(n, prec)
    s.set_state_elements(wf)
    return s


def numpy_marginal(wf, qubits):
    n = int(np.log2(len(wf)))
    p = np.abs(wf) ** 2
    idx = np.arange(len(wf))
    m = np.zeros(len(wf), dtype=np.int64)
    for j, q in enumerate(qubits):
        m |= ((idx >> q) & 1) << j
    return np.bincount(m, weights=p, minlength=1 << len(qubits))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_marginal_probabilities(gpu, prec):
    rng = np.random.default_rng(7)
    for n in (1, 3, 5, 9, 14, 17):
        wf = circuits.random_state(n, seed=n)
        s = upload(wf, prec)
        ref_wf = s.state_elements()
        for k in sorted({0, 1, min(n, 3), min(n, 6), n if n <= 12 else 12}):
            for _ in range(3):
                qs = [int(x) for x in rng.permutation(n)[:k]]
                got = s.marginal_probabilities(qs)
                want = numpy_marginal(ref_wf, qs)
                np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-300)
                np.testing.assert_array_equal(got, s.marginal_probabilities(qs))
        s.free()


def test_marginal_group_bits(gpu):
    """More than 10 qubits: the high ones select CTA groups."""
    n = 22
    wf = circuits.random_state(n, seed=3)
    s = upload(wf)
    for qs in ([21, 0, 20, 1, 19, 2, 18, 3, 17, 4, 16, 5, 15, 6],
               list(range(n - 1, n - 21, -1)),
               [3, 11, 4, 12, 5, 13, 6, 14, 7, 15, 8, 16]):
        got = s.marginal_probabilities(qs)
        want = numpy_marginal(wf, qs)
        np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-300)
        assert abs(got.sum() - 1.0) < 1e-12
    with pytest.raises(Exception):
        s.marginal_probabilities([0, 0])
    with pytest.raises(Exception):
        s.marginal_probabilities(list(range(21)))
    s.free()


def oracle_trials(oracle, wf, qubits, ntrials, draws, compiled=False):
    """Per trial: a fresh copy, then measure each entry in order."""
    out, used = [], 0
    for _ in range(ntrials):
        w = wf.copy()
        row = []
        for q in qubits:
            if q == -1:
                row.append(0)
                continue
            if compiled:
                b, _ = oracle.measure_compiled(w, q, draws[used])
                used += 1
            else:
                b, u, _ = oracle.measure(w, q, draws[used])
                used += int(u)
            row.append(b)
        out.append(row)
    return np.array(out, dtype=np.uint8), used


@pytest.mark.parametrize("compiled", [False, True])
def test_measure_sequence_matches_oracle(gpu, oracle, compiled):
    n = 10
    wf = circuits.random_state(n, seed=11)
    # a qubit that is certainly 0 (p1 = 0: no draw in the interpreted rule)
    wf = wf.reshape(-1)
    idx = np.arange(len(wf))
    wf[(idx >> 7) & 1 == 1] = 0
    wf /= np.linalg.norm(wf)
    s = upload(wf)
    qubits = [3, 0, 7, 9, -1, 3, 5, 7, 2]
    ntrials = 300
    r = random.Random(5)
    draws = [r.random() for _ in range(ntrials * len(qubits))]
    bits, used = s.measure_sequence(qubits, draws, ntrials, compiled=compiled)
    want, want_used = oracle_trials(oracle, wf, qubits, ntrials, draws, compiled)
    np.testing.assert_array_equal(bits, want)
    assert used == want_used
    # the state is untouched
    np.testing.assert_array_equal(s.state_elements(), wf)
    with pytest.raises(Exception):
        s.measure_sequence(qubits, draws[:10], ntrials, compiled=compiled)
    s.free()


def test_multishot_measure_all_and_subset(gpu, oracle):
    prog = "H 0\nCNOT 0 1\nRX(0.9) 2\nCNOT 2 3\nRY(1.3) 4\nH 5\nCZ 5 4"
    n = 6
    gs = [(a.matrix, a.qubits) for a in Q.parse(prog).instructions]
    wf = oracle.zero_state(n)
    for m, qs in gs:
        oracle.apply_matrix_operator(wf, m, qs)
    # all qubits (a permutation, plus a repeat): the measure-all path
    qubits = [5, 4, 3, 2, 1, 0, 2]
    r1 = random.Random(9)
    got = api.perform_multishot_measure(prog, n, qubits, 200, rng=r1)
    r2 = random.Random(9)
    want = []
    for _ in range(200):
        idx = oracle.sample_bisect(wf, r2.random())
        want.append([(idx >> q) & 1 for q in qubits])
    assert got == want
    assert r1.random() == r2.random()
    # a subset: sequential measurement on each reload
    qubits = [4, 1, 0, 4]
    r1 = random.Random(10)
    got = api.perform_multishot_measure(prog, n, qubits, 300, rng=r1)
    r2 = random.Random(10)
    draws = [r2.random() for _ in range(300 * len(qubits))]
    want, used = oracle_trials(oracle, wf, qubits, 300, draws)
    assert got == want.tolist()
    r3 = random.Random(10)
    for _ in range(used):
        r3.random()
    assert r1.random() == r3.random()
    # relabeling: qubit 9 is not in the relabeling (unused -> 0)
    got = api.perform_multishot_measure(prog, n, [4, 9], 5, relabeling=[0, 1, 2, 3, 9, 5],
                                        rng=random.Random(1))
    assert all(len(t) == 2 for t in got)
    assert api.perform_multishot_measure(prog, n, [], 5) == []
    assert api.perform_multishot_measure(prog, n, [1], 0) == []


@pytest.mark.parametrize("compile_mode", [False, True])
def test_multishot_fast_path_equals_trial_runs(gpu, compile_mode):
    prog = ("DECLARE ro BIT[4]\nDECLARE aux BIT[2]\nH 0\nCNOT 0 1\nRX(0.7) 2\nRY(2.1) 3\n"
            "CZ 2 3\nMEASURE 0 ro[0]\nMEASURE 1 ro[1]\nMEASURE 2 ro[2]\nMEASURE 3 ro[3]\n")
    addresses = {"ro": True, "aux": [1]}
    for n in (4, 6):
        got = api.perform_multishot(prog, n, addresses, 250, rng=random.Random(3),
                                    compile=compile_mode)
        qvm = PureStateQVM(n, seed=None, compile=compile_mode)
        qvm.rng = random.Random(3)
        qvm.load_program(prog)
        want = {"ro": [], "aux": []}
        for _ in range(250):
            qvm.reset_quantum_state()
            qvm.run()
            want["ro"].append(list(qvm.memory["ro"]))
            want["aux"].append([qvm.memory["aux"][1]])
        qvm.free()
        assert got == want, (n, compile_mode)
        # Bell pair: ro[0] == ro[1] on every trial
        assert all(t[0] == t[1] for t in got["ro"])
    # a gate after a measurement takes the trial-by-trial path
    prog2 = "DECLARE ro BIT[2]\nH 0\nMEASURE 0 ro[0]\nCNOT 0 1\nMEASURE 1 ro[1]\n"
    got = api.perform_multishot(prog2, 2, {"ro": True}, 50, rng=random.Random(4))
    assert all(t[0] == t[1] for t in got["ro"])
    assert api.perform_multishot(prog2, 2, {}, 50) == {}
    with pytest.raises(ValueError):
        api.perform_multishot(prog2, 2, {"ro": [-1]}, 5)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_expectation(gpu, oracle, prec):
    prep = "H 0\nCNOT 0 1\nRY(0.3) 2\nRX(1.1) 3\nCNOT 3 2"
    ops = ["Z 0", "Z 0\nZ 1", "X 2", "Y 3\nZ 2", "X 0\nX 1", "I 3"]
    n = 4
    got = api.perform_expectation(prep, ops, n, precision=prec)
    wf = oracle.zero_state(n)
    for a in Q.parse(prep).instructions:
        oracle.apply_matrix_operator(wf, a.matrix, a.qubits)
    want = []
    for op in ops:
        w = wf.copy()
        for a in Q.parse(op).instructions:
            oracle.apply_matrix_operator(w, a.matrix, a.qubits)
        want.append(np.vdot(wf, w).real)
    tol = 1e-13 if prec == "fp64" else 1e-6
    np.testing.assert_allclose(got, want, atol=tol)
    assert api.perform_expectation(prep, [], n) == []


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_wire_octets(gpu, prec):
    for n in (1, 6, 13, 23):
        wf = circuits.random_state(n, seed=n)
        s = upload(wf, prec)
        amps = s.state_elements()
        assert s.wavefunction_octets() == amps.astype(">c16").tobytes()
        probs = np.frombuffer(s.probabilities_octets(), dtype=">f8")
        np.testing.assert_allclose(probs, s.probabilities(), rtol=2e-16 if prec == "fp64" else 1e-15,
                                   atol=0)
        s.free()
    qvm = api.perform_wavefunction("H 0\nCNOT 0 1", 2)
    raw = np.frombuffer(api.wavefunction_octets(qvm), dtype=">c16")
    np.testing.assert_allclose(raw, [2 ** -0.5, 0, 0, 2 ** -0.5], atol=1e-15)
    qvm.free()
