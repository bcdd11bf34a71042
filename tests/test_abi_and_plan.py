"""CPU tests of the C-ABI library: it loads, exports every declared entry
point, validates arguments, and its planner (gate fusion + tiling) is
correct -- checked by executing plan descriptions with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from qvm_gb300 import circuits, gates
from qvm_gb300 import _lib as L
from qvm_gb300.state import Program, state_bytes

from .plan_emulator import run_description

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "qvmgpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qvmg_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(qvmlib):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(qvmlib, n), f"libqvmgpu.so does not export {n}"


def test_binding_covers_header(qvmlib):
    assert set(declared_functions()) == set(L.SIGNATURES)


def test_abi_version_and_sizes(qvmlib):
    assert qvmlib.qvmg_abi_version() == 1
    b64 = state_bytes(20, "fp64")
    b32 = state_bytes(20, "fp32")
    assert b64 >= 16 * 2 ** 20 and b32 >= 8 * 2 ** 20
    assert b64 - 16 * 2 ** 20 == b32 - 8 * 2 ** 20  # same scratch
    assert qvmlib.qvmg_state_bytes(0, 0) == 0
    assert qvmlib.qvmg_state_bytes(35, 0) == 0
    assert qvmlib.qvmg_state_bytes(10, 7) == 0


def test_program_argument_validation(qvmlib):
    p = Program()
    with pytest.raises(L.QVMGError, match="repeated qubit"):
        p.add_dense(np.eye(4), [1, 1])
    with pytest.raises(L.QVMGError, match="outside"):
        p.add_dense(np.eye(64), [0, 1, 2, 3, 4, 5])
    with pytest.raises(L.QVMGError, match="not a permutation"):
        p.add_permutation([0, 0], [3])
    p.add_dense(gates.gate_matrix("H"), [3])
    with pytest.raises(L.QVMGError, match="beyond"):
        p.plan(3, "fp64", fused=True)
    with pytest.raises(L.QVMGError, match="fusion width"):
        p.plan(8, "fp64", fused=True, fusion_width=9)
    assert p.num_ops() == 1


def _program(gs):
    p = Program()
    for m, qs in gs:
        p.add_dense(m, qs)
    return p


def _oracle_run(oracle, n, gs, init):
    wf = init.copy()
    for m, qs in gs:
        oracle.apply_matrix_operator(wf, m, qs)
    return wf


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("fw,tile", [(1, 0), (2, 0), (3, 6), (4, 9), (5, 10), (2, 7), (2, 12),
                                     (2, 13)])
def test_fused_plan_equals_circuit(oracle, prec, fw, tile):
    n = 14
    for name, gs in [("su", circuits.random_su_circuit(n, depth=4, seed=fw * 7 + tile)),
                     ("layers", circuits.random_layers(n, layers=3, seed=5)),
                     ("qft", circuits.qft(n))]:
        init = circuits.random_state(n, seed=9)
        want = _oracle_run(oracle, n, gs, init)
        p = _program(gs)
        for reg in (False, True):
            p.set_register_stages(reg)
            st = p.plan(n, prec, fused=True, fusion_width=fw, tile_qubits=tile)
            got = run_description(oracle, p.describe(), init.copy())
            assert np.max(np.abs(got - want)) < 1e-12, (name, reg, st)
            assert st["source_ops"] == len(gs)


@pytest.mark.parametrize("fw,tile", [(2, 0), (4, 0), (2, 11), (4, 12), (1, 13)])
def test_tensor_core_plan_equals_circuit(oracle, fw, tile):
    """FP32 tensor-core planning: the pass-local merge into blocks of <= 4
    tile bits and the split TF32 operand, executed on the oracle, equal the
    unfused circuit to the hi + lo precision (~2^-22 relative per block)."""
    n = 16
    for name, gs in [("su", circuits.random_su_circuit(n, depth=5, seed=fw + tile)),
                     ("layers", circuits.random_layers(n, layers=3, seed=6)),
                     ("qft", circuits.qft(n))]:
        init = circuits.random_state(n, seed=3)
        want = _oracle_run(oracle, n, gs, init)
        p = _program(gs)
        p.set_tensor_cores(True)
        st = p.plan(n, "fp32", fused=True, fusion_width=fw, tile_qubits=tile)
        d = p.describe()
        tcs = [op for ps in d["passes"] if ps["kind"] == "tile" for op in ps["ops"]
               if op["kind"] == "tc"]
        if name != "qft":
            assert tcs, name  # the random circuits produce 3-/4-qubit blocks
        for op in tcs:
            assert 3 <= len(op["pos"]) <= 4
        got = run_description(oracle, d, init.copy())
        assert np.max(np.abs(got - want)) < 2e-6, (name, st)
        # FP64 plans never use the tensor cores
        p.plan(n, "fp64", fused=True, fusion_width=fw, tile_qubits=tile)
        assert not any(op["kind"] == "tc" for ps in p.describe()["passes"]
                       if ps["kind"] == "tile" for op in ps["ops"])


def test_plain_plan_equals_circuit(oracle):
    n = 9
    gs = circuits.qft(n) + circuits.random_layers(n, layers=2, seed=2)
    init = circuits.random_state(n, seed=4)
    want = _oracle_run(oracle, n, gs, init)
    p = _program(gs)
    st = p.plan(n, "fp64", fused=False)
    got = run_description(oracle, p.describe(), init.copy())
    assert np.max(np.abs(got - want)) < 1e-12
    # QFT: the CPHASE chain after each H is folded into phase passes
    assert st["diag_passes"] >= 1 and st["passes"] < len(gs)


def test_register_stages_cover_their_ops():
    """Every op of a register stage lies in the stage's slots, stages cover
    the pass's ops in order, and the FP32 13-qubit tile uses 5 slots."""
    n = 22
    gs = circuits.random_su_circuit(n, depth=6, seed=4) + circuits.qft(n)
    p = _program(gs)
    p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    assert all(ps.get("R", 0) == 0 for ps in p.describe()["passes"])  # off by default
    p.set_register_stages(True)
    p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=13)
    d = p.describe()
    nreg = 0
    for ps in d["passes"]:
        if ps["kind"] != "tile":
            continue
        assert ps["R"] == 5
        nxt = 0
        for st in ps["stages"]:
            assert st["first"] == nxt
            nxt += st["count"]
            if st["reg"]:
                nreg += 1
                assert len(st["slots"]) == 5
                for op in ps["ops"][st["first"]:st["first"] + st["count"]]:
                    assert op["kind"] == "dense" and len(op["pos"]) <= 2
                    assert set(op["pos"]) <= set(st["slots"])
                    assert op["pos"] == sorted(op["pos"])
        assert nxt == len(ps["ops"])
    assert nreg > 0
    p.plan(n, "fp64", fused=True, fusion_width=2, tile_qubits=12)
    assert all(ps.get("R", 0) == 0 for ps in p.describe()["passes"])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_tile_passes_fit_shared_memory(prec):
    """Large QFTs put many ops into a pass: every pass must still fit the
    227 KiB shared-memory limit of one CTA.  Shared memory holds the tile,
    the row offsets, the dense/tensor-core op data and the descriptors;
    diagonal tables are read from global memory."""
    csz = 16 if prec == "fp64" else 8
    for n in (21, 25, 30):
        p = _program(circuits.qft(n))
        p.plan(n, prec, fused=True, fusion_width=2)
        for ps in p.describe()["passes"]:
            if ps["kind"] != "tile":
                continue
            t, L = ps["t"], ps["L"]
            nd = sum(len(o["data"]) for o in ps["ops"] if o["kind"] not in ("perm", "diag"))
            rows = ((1 << (t - L)) + 1) & ~1
            smem = (1 << t) * csz + rows * 8 + nd * csz + len(ps["ops"]) * 128 + \
                len(ps["stages"]) * 80
            assert smem <= 227 * 1024, (n, smem)


def test_fusion_reduces_passes():
    n = 30
    gs = circuits.random_su_circuit(n, depth=20, seed=3)
    p = _program(gs)
    plain = p.plan(n, "fp64", fused=False)
    fused = p.plan(n, "fp32", fused=True, fusion_width=2)
    assert plain["passes"] == len(gs)
    # every SU(2) is absorbed into an SU(4) of the same layer
    assert fused["fused_blocks"] <= len(gs) // 2
    assert fused["passes"] * 5 < plain["passes"]


def test_plan_with_permutations_and_diagonals(oracle):
    n = 10
    rng = np.random.default_rng(1)
    p = Program()
    init = circuits.random_state(n, seed=1)
    want = init.copy()
    for i in range(60):
        r = rng.integers(3)
        qs = [int(x) for x in rng.choice(n, int(rng.integers(1, 4)), replace=False)]
        k = len(qs)
        if r == 0:
            perm = rng.permutation(1 << k)
            p.add_permutation(perm, qs)
            oracle.apply_permutation(want, perm, qs)
        elif r == 1:
            d = np.exp(1j * rng.uniform(0, 6, 1 << k))
            p.add_diagonal(d, qs)
            oracle.apply_matrix_operator(want, np.diag(d), qs)
        else:
            m = gates.haar_unitary(rng, 1 << k)
            p.add_dense(m, qs)
            oracle.apply_matrix_operator(want, m, qs)
    for fused in (False, True):
        p.plan(n, "fp32", fused=fused, fusion_width=3, tile_qubits=7)
        got = run_description(oracle, p.describe(), init.copy())
        assert np.max(np.abs(got - want)) < 1e-12
