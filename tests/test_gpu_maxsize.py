"""States at the ABI's maximum width, QVMG_MAX_QUBITS = 34: amplitude indices
above 2^32 in every kernel on the path (tile passes, plain gates, the
probability and marginal reductions, the two-level sampler, collapse).

Nothing is downloaded (a 34-qubit state is 128 GiB in FP32, 256 GiB in
FP64): the checks are device reductions, sampled indices and measured bits.

- FP32, 34 qubits: a random SU(2)/SU(4) circuit and its inverse, fused into
  tile passes, return the state to |0...0>.
- FP64, 34 qubits: H, CNOT and a measurement on the top and middle qubits,
  plain kernels.  If the device cannot hold 256 GiB, state creation must fail
  with QVMG_E_NOMEM and leave the library usable.
"""
import numpy as np
import pytest

from qvm_gb300 import CudaPureState, Program, circuits, gates
from qvm_gb300 import _lib as L

pytestmark = pytest.mark.gpu

N_MAX = 34


def _inverse(gs):
    return [(gates.dagger(m), qs) for m, qs in reversed(gs)]


def test_max_width_constant():
    assert N_MAX == 34  # include/qvmgpu.h QVMG_MAX_QUBITS


def test_fp32_34_qubits_circuit_and_inverse(gpu):
    n = N_MAX
    gs = circuits.random_su_circuit(n, depth=3, seed=5)
    fwd, inv = Program(), Program()
    fwd.add_gates(gs)
    inv.add_gates(_inverse(gs))
    fwd.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    inv.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    s = CudaPureState(n, "fp32")
    try:
        fwd.run(s, fused=True)
        assert abs(s.norm() - 1.0) < 1e-5
        top = s.marginal_probabilities([30, 31, 32, 33])
        assert abs(top.sum() - 1.0) < 1e-5
        assert top.max() < 0.5  # spread over the top qubits
        inv.run(s, fused=True)
        assert abs(s.norm() - 1.0) < 1e-5
        for q in (0, 5, 13, 17, 31, 32, 33):
            assert s.excited_probability(q) < 1e-5, q
        top = s.marginal_probabilities([30, 31, 32, 33])
        assert top[0] > 1 - 1e-5
        draws = np.random.default_rng(3).random(64) * 0.999
        assert (s.sample(draws) == 0).all()
    finally:
        s.free()
        fwd.free()
        inv.free()


def test_fp64_34_qubits_bell_pair_and_measurement(gpu):
    n = N_MAX
    try:
        s = CudaPureState(n, "fp64")
    except L.QVMGError as e:
        assert e.args[0] == 3, e  # QVMG_E_NOMEM
        with CudaPureState(20, "fp64") as small:  # the library is still usable
            assert abs(small.norm() - 1.0) < 1e-12
        pytest.skip(f"256 GiB FP64 state does not fit this device: {e}")
    try:
        s.apply_matrix(gates.gate_matrix("H"), [33])
        s.apply_matrix(gates.gate_matrix("CNOT"), [16, 33])  # CNOT 33 16 as a nat-tuple
        assert abs(s.excited_probability(33) - 0.5) < 1e-12
        assert abs(s.excited_probability(16) - 0.5) < 1e-12
        assert s.excited_probability(0) < 1e-15
        idx = s.sample(np.array([0.25, 0.75]))
        assert [int(i) for i in idx] == [0, (1 << 33) | (1 << 16)]
        bit, used, p1 = s.measure(33, 0.3)  # bit 1 iff draw <= P(q=1)
        assert bit == 1 and used and abs(p1 - 0.5) < 1e-12
        assert abs(s.excited_probability(16) - 1.0) < 1e-12
        assert abs(s.norm() - 1.0) < 1e-12
    finally:
        s.free()
