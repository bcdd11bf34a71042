"""Oracle parity at the workloads' full sizes.

The CPU oracle (the reference's apply-matrix-operator and CDF sampler,
restated in C) ran these circuits once at full size; its states are pinned
by fingerprints committed under ``golden/`` (made by
``golden/make_fullsize.py``; see ``fullsize_common.py``):

- the 28-qubit QFT in FP64 on the seeded complex-Gaussian state, on the
  plain kernels and on the fused double-float tiles: 1e-12 per amplitude;
- the first full layer of the 30-qubit random SU(2)/SU(4) circuit: plain
  FP64 at 1e-12 per amplitude, and 4096 FP64 samples identical to the
  oracle's on the same draws except the draws the oracle side marks as lying
  on a CDF boundary; fused FP32 within fidelity 1 - 1e-6 of plain FP64.
"""
import os

import numpy as np
import pytest

from qvm_gb300 import CudaPureState, Program, circuits
from tests import fullsize_common as F

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


@pytest.mark.parametrize("mode", ["plain", "fused"])
def test_qft28_fp64_matches_oracle(gpu, mode):
    fx = _load("qft28_fp64.npz")
    n = int(fx["n"])
    s = CudaPureState(n, "fp64")
    s.set_state_elements(circuits.random_state(n, seed=int(fx["state_seed"])))
    p = Program()
    p.add_gates(circuits.qft(n))
    fused = mode == "fused"
    if fused:
        p.plan(n, "fp64", fused=True, fusion_width=2, tile_qubits=12)
    p.run(s, fused=fused)
    got = s.state_elements()
    s.free()
    p.free()
    amp_err, sum_err = F.compare(got, n, fx)
    assert amp_err < 1e-12, amp_err
    assert sum_err < 1e-12, sum_err


def _layer(fx):
    mats, kq, qubits = fx["mats"], fx["kq"], fx["qubits"]
    gates, mo, qo = [], 0, 0
    for k in kq:
        d = 1 << int(k)
        gates.append((mats[mo:mo + d * d].reshape(d, d), [int(q) for q in qubits[qo:qo + k]]))
        mo += d * d
        qo += int(k)
    return gates


def test_random30_first_layer_matches_oracle(gpu):
    fx = _load("random30_layer1.npz")
    n = int(fx["n"])
    gates = _layer(fx)
    assert len(gates) == n + n // 2
    p = Program()
    p.add_gates(gates)
    s64 = CudaPureState(n, "fp64")
    p.run(s64, fused=False)
    # 4096 samples on the oracle's draws, CDF rule (smallest i with C(i) >= p)
    draws = np.asarray(fx["draws"], dtype=np.float64)
    got_shots = s64.sample(draws, rule="cdf")
    want = np.asarray(fx["shots"], dtype=np.uint64)
    exempt = np.asarray(fx["exempt"], dtype=bool)
    bad = np.nonzero((got_shots != want) & ~exempt)[0]
    assert len(bad) == 0, (len(bad), bad[:8])
    # fused FP32 against the device's plain FP64 state
    p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    s32 = CudaPureState(n, "fp32")
    p.run(s32, fused=True)
    f, err = s64.fidelity(s32)
    s32.free()
    assert f >= 1 - 1e-6, f
    got = s64.state_elements()
    s64.free()
    p.free()
    amp_err, sum_err = F.compare(got, n, fx)
    assert amp_err < 1e-12, amp_err
    assert sum_err < 1e-12, sum_err
