"""GPU: the PureStateQVM API on Quil programs from the reference's tests."""
import numpy as np
import pytest

from qvm_gb300 import PureStateQVM, run_program

from .test_oracle_kat import KATS

pytestmark = pytest.mark.gpu

MODES = [dict(compile=False, fused=False), dict(compile=True, fused=False),
         dict(compile=True, fused=True)]


@pytest.mark.parametrize("mode", MODES)
def test_gate_programs(gpu, mode):
    k = KATS["gate_programs"]
    for c in k["cases"]:
        qvm = run_program(c["n"], c["program"], **mode)
        p = np.abs(qvm.amplitudes[c["index"]]) ** 2
        assert abs(p - c["value"]) < k["tolerance"], c["name"]
        qvm.free()


@pytest.mark.parametrize("mode", MODES)
def test_hadamard_and_bell(gpu, mode):
    """tests/gate-tests.lisp:13-26, :75-89"""
    for n in range(1, 11):
        h = "\n".join(f"H {q}" for q in range(n))
        qvm = run_program(n, h, **mode)
        assert np.all(np.abs(np.abs(qvm.amplitudes) ** 2 - 2.0 ** -n) < 1e-4)
        qvm.free()
        bell = "H 0\n" + "\n".join(f"CNOT 0 {i}" for i in range(1, n))
        qvm = run_program(n, bell, **mode)
        a = qvm.amplitudes
        assert abs(abs(a[0]) ** 2 - 0.5) < 1e-4 and abs(abs(a[-1]) ** 2 - 0.5) < 1e-4
        qvm.free()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("key", ["simple_measurements", "simple_measurements_with_swap",
                                 "cheeky_measurements_with_swap"])
def test_deterministic_measurements(gpu, mode, key):
    c = KATS[key]
    from qvm_gb300 import quil
    prog = quil.parse(c["program"])
    qvm = run_program(prog.qubits_needed(), prog, seed=3, **mode)
    assert [qvm.memory_ref("ro", i) for i in range(3)] == c["ro"]
    qvm.free()


def test_swap_direct(gpu):
    """tests/gate-tests.lisp:91-103"""
    qvm = PureStateQVM(2)
    qvm.load_program("X 0").run()
    assert abs(abs(qvm.amplitudes[1]) ** 2 - 1) < 1e-4
    qvm.load_program("SWAP 0 1").run()
    assert abs(abs(qvm.amplitudes[2]) ** 2 - 1) < 1e-4
    qvm.free()


def test_interpreted_equals_compiled_ordering(gpu):
    """tests/gate-tests.lisp:28-44"""
    c = KATS["qubit_ordering_compiled"]
    a = run_program(c["n"], c["program"]).amplitudes
    b = run_program(c["n"], c["program"], compile=True, fused=True).amplitudes
    np.testing.assert_allclose(a, b, atol=1e-12)


def test_unit_norm_after_measurements(gpu):
    """tests/measurement-tests.lisp:88-109"""
    for n in range(5, 16):
        prog = "\n".join(f"H {q}\nMEASURE {q}" for q in range(n))
        for mode in MODES:
            qvm = run_program(n, prog, seed=n, **mode)
            assert abs(qvm.state.norm() - 1) < 1e-12
            qvm.free()


@pytest.mark.parametrize("compile", [False, True])
def test_statistical_rotation_measurements(gpu, compile):
    """tests/measurement-tests.lisp:111-182 (quarter rotation, 20000 trials)."""
    one = np.sin(np.pi / 4 / 2) ** 2
    qvm = PureStateQVM(2, seed=11, compile=compile)
    qvm.load_program("DECLARE ro BIT\nI 1\nRX(pi/4) 0\nMEASURE 0 ro[0]\nRESET")
    trials, ones = 20000, 0
    for _ in range(trials):
        qvm.reset_classical_memory()
        qvm.reset_quantum_state()
        qvm.run()
        ones += qvm.memory_ref("ro", 0)
    assert abs(ones / trials - one) < 0.02
    qvm.free()


def test_out_of_range_measure(gpu):
    """tests/measurement-tests.lisp:265-269"""
    qvm = PureStateQVM(1)
    with pytest.raises(ValueError):
        qvm.measure(1)
    with pytest.raises(ValueError):
        qvm.measure(-1)
    qvm.measure(0)
    qvm.free()


def test_same_seed_same_results(gpu):
    prog = "DECLARE ro BIT[6]\n" + "\n".join(f"H {q}\nRX(0.3) {q}" for q in range(6)) + \
        "\n" + "\n".join(f"MEASURE {q} ro[{q}]" for q in range(6))
    outs = []
    for mode in MODES:
        for _ in range(2):
            qvm = run_program(6, prog, seed=42, **mode)
            outs.append((mode["compile"], tuple(qvm.memory["ro"])))
            qvm.free()
    # identical within a mode (same seed, same draws)
    assert outs[0][1] == outs[1][1] and outs[2][1] == outs[3][1] and outs[4][1] == outs[5][1]
    # compiled runs (measure-all chain, one draw) agree with each other
    assert outs[2][1] == outs[4][1]
