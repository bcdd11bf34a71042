"""GPU parity: per-gate kernels and programs against the CPU oracle.

FP64 results must match the oracle within 1e-12 (absolute, per amplitude);
FP32 within 2e-6 absolute per amplitude on normalised states and fidelity
>= 1 - 1e-6.
"""
import itertools
import os

import numpy as np
import pytest

from qvm_gb300 import CudaPureState, Program, circuits, gates

from .plan_emulator import _apply_table

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-6


def upload(wf, prec="fp64"):
    n = int(np.log2(len(wf)))
    s = CudaPureState(n, prec)
    s.set_state_elements(wf)
    return s


def tol(prec):
    return TOL64 if prec == "fp64" else TOL32


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_upload_download_roundtrip(gpu, prec):
    for n in (1, 2, 5, 13, 17):
        wf = circuits.random_state(n, seed=n)
        s = upload(wf, prec)
        got = s.state_elements()
        if prec == "fp64":
            np.testing.assert_array_equal(got, wf)
        else:
            np.testing.assert_array_equal(got, wf.astype(np.complex64).astype(np.complex128))
        s.set_to_zero_state()
        z = s.state_elements()
        assert z[0] == 1 and np.count_nonzero(z) == 1
        s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_dense_all_tuples_small(gpu, oracle, prec):
    """Every ordered qubit tuple of width 1..3 on a 6-qubit state, random
    unitaries (the AVX-kernel-vs-Lisp style of tests/qvm-avx-intrinsics.lisp)."""
    n = 6
    rng = np.random.default_rng(1)
    for k in (1, 2, 3):
        for qs in itertools.permutations(range(n), k):
            m = gates.haar_unitary(rng, 1 << k)
            wf = circuits.random_state(n, seed=int(rng.integers(1 << 30)))
            s = upload(wf, prec)
            s.apply_matrix(m, list(qs))
            want = oracle.apply_matrix_operator(wf.copy(), m, list(qs))
            assert np.max(np.abs(s.state_elements() - want)) < tol(prec), (k, qs)
            s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_dense_wide_and_real(gpu, oracle, prec, k):
    n = 16
    rng = np.random.default_rng(k)
    for trial in range(6):
        qs = [int(x) for x in rng.choice(n, k, replace=False)]
        if trial % 2:
            m = np.real(gates.haar_unitary(rng, 1 << k)) + 0j  # real-matrix kernel
        else:
            m = gates.haar_unitary(rng, 1 << k)
        wf = circuits.random_state(n, seed=trial)
        s = upload(wf, prec)
        s.apply_matrix(m, qs)
        want = oracle.apply_matrix_operator(wf.copy(), m, qs)
        scale = max(1.0, np.max(np.abs(m)) * 4)
        assert np.max(np.abs(s.state_elements() - want)) < tol(prec) * scale
        s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_permutation_and_diagonal(gpu, oracle, prec):
    n = 12
    rng = np.random.default_rng(3)
    for trial in range(30):
        k = int(rng.integers(1, 6))
        qs = [int(x) for x in rng.choice(n, k, replace=False)]
        wf = circuits.random_state(n, seed=trial)
        s = upload(wf, prec)
        perm = rng.permutation(1 << k)
        s.apply_permutation(perm, qs)
        want = oracle.apply_permutation(wf.copy(), perm, qs)
        got = s.state_elements()
        if prec == "fp64":
            np.testing.assert_array_equal(got, want)  # pure data movement: bit-exact
        else:
            assert np.max(np.abs(got - want)) < TOL32
        kd = int(rng.integers(1, 11))
        qd = [int(x) for x in rng.choice(n, kd, replace=False)]
        d = np.exp(1j * rng.uniform(0, 2 * np.pi, 1 << kd))
        s.apply_diagonal(d, qd)
        _apply_table(want, qd, d)
        assert np.max(np.abs(s.state_elements() - want)) < tol(prec)
        s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_diagonal_required_qubits(gpu, oracle, prec):
    """Diagonal passes visit only the amplitudes whose required qubits (held
    by every table, with every entry for their 0 value exactly 1) are set.
    Cases: CZ with qubit 0 (the FP32 single-amplitude path), CPHASE, a
    3-qubit controlled phase, unit entries that make no qubit required, one
    required qubit beside one that is not, and a CPHASE chain with a lone CZ
    through the program's plain plan."""
    n = 12
    rng = np.random.default_rng(21)
    ph = lambda: np.exp(1j * rng.uniform(0.1, 2 * np.pi - 0.1))  # never exactly 1
    cases = [
        ([0, 5], np.array([1, 1, 1, -1], dtype=complex)),                  # CZ: {0, 5}
        ([9, 3], np.array([1, 1, 1, ph()])),                               # CPHASE: {3, 9}
        ([11, 6, 1], np.array([1] * 7 + [ph()])),                          # {1, 6, 11}
        ([2, 7], np.array([ph(), 1, 1, ph()])),                            # none
        ([4, 8], np.array([1, ph(), 1, ph()])),                            # {4}
        ([10], np.array([1, ph()])),                                       # PHASE: {10}
    ]
    wf = circuits.random_state(n, seed=5)
    s = upload(wf, prec)
    want = wf.copy()
    for qs, d in cases:
        s.apply_diagonal(d, qs)
        _apply_table(want, qs, d)
        assert np.max(np.abs(s.state_elements() - want)) < tol(prec), (qs, prec)
    s.free()
    # the same through a program: a CPHASE chain on target 9 (one table pass),
    # then a lone CZ 0 11, each separated by an H so that they stay separate passes
    gs = [(gates.gate_matrix("H"), [9])]
    gs += [(gates.gate_matrix("CPHASE", np.pi / 2 ** (9 - j)), [9, j]) for j in range(9)]
    gs += [(gates.gate_matrix("H"), [3]), (gates.gate_matrix("CZ"), [11, 0]),
           (gates.gate_matrix("H"), [0])]
    want = _oracle(oracle, gs, n, init=wf)
    got = _run_program(gs, n, prec, fused=False, init=wf).state_elements()
    assert np.max(np.abs(got - want)) < tol(prec) * 4


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_standard_gates(gpu, oracle, prec):
    """Every standard gate through apply_dense (which routes permutation and
    diagonal matrices to their kernels)."""
    n = 7
    rng = np.random.default_rng(4)
    wf = circuits.random_state(n, seed=4)
    s = upload(wf, prec)
    want = wf.copy()
    for name, (npar, _) in gates.STANDARD_GATES.items():
        m = gates.gate_matrix(name, *rng.uniform(-3, 3, npar))
        k = int(np.log2(m.shape[0]))
        qs = [int(x) for x in rng.choice(n, k, replace=False)]
        s.apply_matrix(m, qs)
        oracle.apply_matrix_operator(want, m, qs)
    assert np.max(np.abs(s.state_elements() - want)) < tol(prec) * 10
    s.free()


def _run_program(gs, n, prec, fused, init=None, fw=2, tile=0, reg=False, tc=False):
    p = Program()
    p.add_gates(gs)
    p.set_register_stages(reg)
    p.set_tensor_cores(tc)
    if fused:
        p.plan(n, prec, fused=True, fusion_width=fw, tile_qubits=tile)
    s = CudaPureState(n, prec)
    if init is not None:
        s.set_state_elements(init)
    p.run(s, fused=fused)
    return s


def _oracle(oracle, gs, n, init=None):
    wf = oracle.zero_state(n) if init is None else init.copy()
    for m, qs in gs:
        oracle.apply_matrix_operator(wf, m, qs)
    return wf


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("fused", [False, True])
def test_layer_circuit_20q(gpu, oracle, prec, fused):
    """Random RX/RZ + CNOT layer circuit at 20 qubits."""
    n = 20
    gs = circuits.random_layers(n, layers=10, seed=1)
    want = _oracle(oracle, gs, n)
    s = _run_program(gs, n, prec, fused)
    got = s.state_elements()
    assert np.max(np.abs(got - want)) < tol(prec)
    if prec == "fp32":
        f = abs(np.vdot(want, got)) ** 2
        assert f >= 1 - 1e-6
    s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("fused", [False, True])
def test_qft_on_random_state(gpu, oracle, prec, fused):
    n = 16
    gs = circuits.qft(n)
    init = circuits.random_state(n, seed=2)
    want = _oracle(oracle, gs, n, init)
    s = _run_program(gs, n, prec, fused, init=init)
    assert np.max(np.abs(s.state_elements() - want)) < tol(prec)
    s.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("fw,tile", [(1, 0), (2, 0), (2, 10), (3, 12), (4, 11), (5, 13)])
def test_random_su_fused(gpu, oracle, prec, fw, tile):
    n = 18
    gs = circuits.random_su_circuit(n, depth=6, seed=fw + tile)
    want = _oracle(oracle, gs, n)
    s = _run_program(gs, n, prec, True, fw=fw, tile=tile)
    got = s.state_elements()
    assert np.max(np.abs(got - want)) < tol(prec) * 2
    s.free()


@pytest.mark.parametrize("tile", [12, 13])
def test_register_stages(gpu, oracle, tile):
    """FP32 tiles with register stages (16 or 32 amplitudes per thread),
    mixed with shared-memory ops (diagonal, permutation, 3-qubit blocks)."""
    n = 18
    rng = np.random.default_rng(tile)
    gs = circuits.random_su_circuit(n, depth=5, seed=tile) + circuits.qft(n)
    gs += [(gates.gate_matrix("CCNOT"), [int(x) for x in rng.choice(n, 3, replace=False)]),
           (gates.haar_unitary(rng, 8), [int(x) for x in rng.choice(n, 3, replace=False)])]
    gs += circuits.random_layers(n, layers=2, seed=tile)
    want = _oracle(oracle, gs, n)
    s = _run_program(gs, n, "fp32", True, fw=3, tile=tile, reg=True)
    assert np.max(np.abs(s.state_elements() - want)) < 4e-6
    s.free()


@pytest.mark.parametrize("fw,tile", [(2, 13), (4, 13), (4, 12), (3, 11), (5, 13), (5, 14)])
def test_tensor_core_tiles(gpu, oracle, fw, tile):
    """FP32 tiles whose merged 3- to 5-qubit blocks run as tcgen05 bf16x3
    MMAs (hi/lo split operands), mixed with 2-qubit FMA blocks, permutations
    and diagonal tables (14-qubit tiles: a 5-qubit op takes two TMEM batches,
    the first read out into HBM before the second is gathered).  The MMA accumulator rounds toward zero, which shrinks
    the norm by ~1e-7 per block; the comparison is per amplitude (4e-6) and
    as a normalised overlap (1 - 1e-6)."""
    n = 18
    rng = np.random.default_rng(tile + fw)
    gs = circuits.random_su_circuit(n, depth=5, seed=tile) + circuits.qft(n)
    gs += [(gates.gate_matrix("CCNOT"), [int(x) for x in rng.choice(n, 3, replace=False)]),
           (gates.haar_unitary(rng, 8), [int(x) for x in rng.choice(n, 3, replace=False)])]
    gs += circuits.random_layers(n, layers=2, seed=tile)
    want = _oracle(oracle, gs, n)
    s = _run_program(gs, n, "fp32", True, fw=fw, tile=tile, tc=True)
    got = s.state_elements()
    assert np.max(np.abs(got - want)) < 4e-6
    assert abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real >= 1 - 1e-6
    s.free()


def test_tensor_core_pass_diagonal_on_each_tile_bit(gpu, oracle):
    """A 4-qubit block (a tensor-core op) and then an RZ that cannot join it
    (diagonals join blocks of at most two qubits) leave a diagonal op in the
    tensor-core pass.  Gates on qubits 5..12 only give the tile bits 5..12 to
    those qubits, so the RZ walks through every tile bit of the pass.  The
    diagonal op's threads each take a fixed stride of elements; with a
    stride that is not a power of two (a 288-thread team) a phase read once
    per thread would cover elements whose tile bit 8 differs."""
    n = 18
    rng = np.random.default_rng(12)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    for q in range(5, 13):
        others = [x for x in (6, 9, 12, 10) if x != q][:3]
        gs = [(gates.haar_unitary(rng, 16), [q] + others), (gates.gate_matrix("RZ", 0.9), [q])]
        p = Program()
        p.add_gates(gs)
        p.set_tensor_cores(True)
        p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
        (ps,) = p.describe()["passes"]
        assert [op["kind"] for op in ps["ops"]] == ["tc", "diag"], ps["ops"]
        assert ps["ops"][1]["tpos"] == [q] and ps["ops"][1]["req_tile"] == []
        s = CudaPureState(n, "fp32")
        s.set_state_elements(init)
        p.run(s, fused=True)
        want = _oracle(oracle, gs, n, init)
        assert np.max(np.abs(s.state_elements() - want)) < 4e-6, q
        s.free()
        p.free()


def test_tensor_core_tiles_per_cta(gpu, oracle):
    """A tensor-core pass's last op writes its readout into HBM and loads the
    CTA's next tile under its MMAs.  Against the oracle with few and many
    tiles per CTA: 16 qubits (8 tiles, one per CTA: no next tile), 22 qubits
    (512 tiles over 304 CTAs: one or two each) and 26 qubits on a yielding
    state (priority -1: CTAs of 16 tiles)."""
    oracle.set_workers(os.cpu_count() or 1)
    for n, prio, depth in ((16, 0, 6), (22, 0, 4), (26, -1, 2)):
        gs = circuits.random_su_circuit(n, depth=depth, seed=n)
        want = _oracle(oracle, gs, n)
        p = Program()
        p.add_gates(gs)
        p.set_tensor_cores(True)
        p.plan(n, "fp32", fused=True, fusion_width=5, tile_qubits=13)
        assert any(op["kind"] == "tc" for ps in p.describe()["passes"] if ps["kind"] == "tile"
                   for op in ps["ops"])
        s = CudaPureState(n, "fp32")
        s.set_priority(prio)
        p.run(s, fused=True)
        got = s.state_elements()
        assert np.max(np.abs(got - want)) < 4e-6, n
        assert abs(np.vdot(want, got)) ** 2 / np.vdot(got, got).real >= 1 - 1e-6, n
        s.free()
        p.free()


def test_tensor_core_wait_gives_up_and_context_recovers(gpu, oracle):
    """The wait of a tensor-core op for its MMAs is bounded.  With the MMA
    warp told to issue nothing (a test hook: nothing is in flight), the wait
    runs out, the run reports QVMG_E_TIMEOUT through the status word, the
    kernel frees its tensor memory, and the same program then runs correctly
    on the same context."""
    from qvm_gb300 import QVMGError
    from qvm_gb300 import _lib as L
    n = 16
    rng = np.random.default_rng(31)
    gs = [(gates.haar_unitary(rng, 16), [6, 9, 12, 10])]
    p = Program()
    p.add_gates(gs)
    p.set_tensor_cores(True)
    p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    (ps,) = p.describe()["passes"]
    assert [op["kind"] for op in ps["ops"]] == ["tc"]
    init = circuits.random_state(n, seed=32)
    s = CudaPureState(n, "fp32")
    s.set_state_elements(init)
    L.call("qvmg_debug_tc_withhold", 1)
    try:
        with pytest.raises(QVMGError, match="timed out") as err:
            p.run(s, fused=True)
        assert err.value.code == 6  # QVMG_E_TIMEOUT
    finally:
        L.call("qvmg_debug_tc_withhold", 0)
    s.set_state_elements(init)
    p.run(s, fused=True)
    want = _oracle(oracle, gs, n, init)
    assert np.max(np.abs(s.state_elements() - want)) < 4e-6
    s.free()
    p.free()


def test_tensor_core_fidelity_26q(gpu):
    """Fused FP32 with the tensor-core engine vs plain FP64 at 26 qubits."""
    n = 26
    gs = circuits.random_su_circuit(n, depth=20, seed=3)
    s64 = _run_program(gs, n, "fp64", False)
    s32 = _run_program(gs, n, "fp32", True, fw=4, tile=13, tc=True)
    f, err = s64.fidelity(s32)
    assert f >= 1 - 1e-6 and err < 1e-5
    s64.free()
    s32.free()


def test_small_states_all_paths(gpu, oracle):
    """States smaller than a tile row (n = 1..5) in every mode."""
    for n in range(1, 6):
        gs = circuits.random_su_circuit(n, depth=3, seed=n) if n > 1 else [
            (gates.gate_matrix("H"), [0]), (gates.gate_matrix("RZ", 0.3), [0])]
        want = _oracle(oracle, gs, n)
        for prec in ("fp64", "fp32"):
            for fused in (False, True):
                s = _run_program(gs, n, prec, fused)
                assert np.max(np.abs(s.state_elements() - want)) < tol(prec), (n, prec, fused)
                s.free()


def test_fused_fp64_double_float_accuracy(gpu):
    """Fused FP64 tiles compute in double-float (FP32 pairs); against the
    plain FP64 kernels at 24 qubits the amplitudes agree to well inside
    1e-12 and the overlap is 1 to FP64 rounding."""
    n = 24
    gs = circuits.random_su_circuit(n, depth=12, seed=6) + circuits.qft(n)
    plain = _run_program(gs, n, "fp64", False)
    fused = _run_program(gs, n, "fp64", True, fw=2, tile=12)
    f, err = plain.fidelity(fused)
    assert err < 1e-13, err
    assert f > 1 - 1e-13
    plain.free()
    fused.free()


def test_determinism_fp64(gpu):
    n = 20
    gs = circuits.random_su_circuit(n, depth=5, seed=8)
    a = _run_program(gs, n, "fp64", True).state_elements()
    b = _run_program(gs, n, "fp64", True).state_elements()
    np.testing.assert_array_equal(a, b)


def test_fp32_fidelity_26q(gpu):
    """Fused FP32 vs plain FP64 on the device at 26 qubits, depth 20."""
    n = 26
    gs = circuits.random_su_circuit(n, depth=20, seed=3)
    s64 = _run_program(gs, n, "fp64", False)
    s32 = _run_program(gs, n, "fp32", True)
    f, err = s64.fidelity(s32)
    assert f >= 1 - 1e-6
    assert err < 1e-5
    assert abs(s32.norm() - 1) < 1e-5
    s64.free()
    s32.free()
