"""Size-independent properties at the bench's full sizes, where the CPU
oracle would take too long:

- a 30-qubit random circuit followed by its inverse returns the fused FP32
  state to |0...0> (FMA and tensor-core engines), through a device inner
  product (no 16 GB download);
- the 28-qubit FP64 QFT followed by its inverse returns the random input
  state (plain kernels, 1e-12 per amplitude);
- fused FP64 (double-float tiles) and plain FP64 give the same 4096 shots
  for the same draws at 28 qubits.
"""
import numpy as np
import pytest

from qvm_gb300 import CudaPureState, Program, circuits, gates

pytestmark = pytest.mark.gpu


def _inverse(gs):
    return [(gates.dagger(m), qs) for m, qs in reversed(gs)]


def _program(gs, tc=False):
    p = Program()
    p.add_gates(gs)
    p.set_tensor_cores(tc)
    return p


@pytest.mark.parametrize("engine", ["fma", "tc"])
def test_random_circuit_and_inverse_30q(gpu, engine):
    n = 30
    gs = circuits.random_su_circuit(n, depth=20, seed=3)
    fw = 4 if engine == "tc" else 2
    fwd = _program(gs, tc=engine == "tc")
    inv = _program(_inverse(gs), tc=engine == "tc")
    fwd.plan(n, "fp32", fused=True, fusion_width=fw, tile_qubits=13)
    inv.plan(n, "fp32", fused=True, fusion_width=fw, tile_qubits=13)
    s = CudaPureState(n, "fp32")
    zero = CudaPureState(n, "fp32")
    fwd.run(s, fused=True)
    # the forward state is spread out: no basis state dominates
    assert abs(zero.inner(s)) ** 2 < 1e-6
    inv.run(s, fused=True)
    f, _ = zero.fidelity(s)
    assert f >= 1 - 1e-6, f
    s.free()
    zero.free()


def test_qft_roundtrip_28q_fp64(gpu):
    n = 28
    rng = np.random.default_rng(2)
    wf = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    wf /= np.linalg.norm(wf)
    s = CudaPureState(n, "fp64")
    s.set_state_elements(wf)
    q = circuits.qft(n)
    _program(q).run(s, fused=False)
    _program(_inverse(q)).run(s, fused=False)
    back = s.state_elements()
    assert np.max(np.abs(back - wf)) < 1e-12
    s.free()


def test_double_float_tiles_sample_like_plain_fp64_28q(gpu):
    n = 28
    gs = circuits.random_su_circuit(n, depth=8, seed=11)
    plain = CudaPureState(n, "fp64")
    fused = CudaPureState(n, "fp64")
    p = _program(gs)
    p.run(plain, fused=False)
    p.plan(n, "fp64", fused=True, fusion_width=2, tile_qubits=12)
    p.run(fused, fused=True)
    f, err = plain.fidelity(fused)
    assert err < 1e-13 and f > 1 - 1e-13
    draws = np.random.default_rng(5).random(4096)
    assert (plain.sample(draws) == fused.sample(draws)).all()
    plain.free()
    fused.free()
