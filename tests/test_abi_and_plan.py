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


@pytest.mark.parametrize("fw,tile", [(2, 0), (4, 0), (2, 11), (4, 12), (1, 13), (5, 13), (5, 14)])
def test_tensor_core_plan_equals_circuit(oracle, fw, tile):
    """FP32 tensor-core planning: the pass-local merge into blocks of up to
    the fusion width's tile bits (3..5) and the split bf16 operand, executed on the oracle, equal the
    unfused circuit to the hi + lo precision of the block (~2^-17 relative
    per entry)."""
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
        for op in tcs:  # blocks of up to the fusion width's qubits (3..5)
            assert 3 <= len(op["pos"]) <= min(5, max(3, fw))
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


def _required(qubit_lists, tables):
    """Qubits every table holds whose 0 value makes every entry exactly 1."""
    out = []
    for q in qubit_lists[0]:
        ok = True
        for qs, tab in zip(qubit_lists, tables):
            if q not in qs:
                ok = False
                break
            i = qs.index(q)
            for e, (re, im) in enumerate(tab):
                if not (e >> i) & 1 and (re != 1.0 or im != 0.0):
                    ok = False
        if ok:
            out.append(q)
    return sorted(out)[:4]


def _diag_programs():
    rng = np.random.default_rng(12)
    yield 14, circuits.qft(14)
    yield 20, circuits.qft(20)
    gs = []
    for _ in range(40):  # CPHASE / CZ / RZ / dense mixes
        a, b = (int(x) for x in rng.choice(16, 2, replace=False))
        kind = int(rng.integers(4))
        if kind == 0:
            gs.append((gates.gate_matrix("CPHASE", float(rng.uniform(0.1, 3))), [a, b]))
        elif kind == 1:
            gs.append((gates.gate_matrix("CZ"), [a, b]))
        elif kind == 2:
            gs.append((gates.gate_matrix("RZ", float(rng.uniform(0.1, 3))), [a]))
        else:
            gs.append((gates.gate_matrix("H"), [a]))
    yield 16, gs


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_plain_diagonal_required_qubits(prec):
    """A plain diagonal pass visits only the amplitudes with its required
    qubits set; the planner's choice equals a direct check of the tables."""
    for n, gs in _diag_programs():
        p = _program(gs)
        p.plan(n, prec, fused=False)
        for ps in p.describe()["passes"]:
            if ps["kind"] != "diag":
                continue
            qls = [t["qubits"] for t in ps["tables"]]
            tabs = [t["table"] for t in ps["tables"]]
            assert ps["req"] == _required(qls, tabs), ps["req"]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_tile_diagonal_index_layout(prec):
    """A diagonal op inside a tile pass reads its table index from the tile
    index (runs of in-tile bits) and a per-tile constant (out-of-tile bits):
    for random elements and tiles that equals gathering the index from the
    global address; required bits match a direct check of the table."""
    rng = np.random.default_rng(3)
    for n, gs in _diag_programs():
        p = _program(gs)
        p.plan(n, prec, fused=True, fusion_width=2)
        for ps in p.describe()["passes"]:
            if ps["kind"] != "tile":
                continue
            t, L, E = ps["t"], ps["L"], ps["E"]
            tile_of = {q: q for q in range(L)}
            tile_of.update({q: L + e for e, q in enumerate(E)})
            for op in ps["ops"]:
                if op["kind"] != "diag":
                    continue
                pos, tpos = op["pos"], op["tpos"]
                assert tpos == [tile_of.get(q, 255) for q in pos]
                req = _required([pos], [op["data"]])
                assert op["req_tile"] == sorted(tile_of[q] for q in req if q in tile_of)[:4]
                assert op["out_req"] == sum(1 << pos.index(q) for q in req if q not in tile_of)
                for _ in range(64):
                    j = int(rng.integers(1 << t))
                    g = int(rng.integers(1 << n))  # out-of-tile bits of the tile's base
                    for b in range(t):            # the element's in-tile bits
                        q = b if b < L else E[b - L]
                        g = (g & ~(1 << q)) | (((j >> b) & 1) << q)
                    want = sum(((g >> q) & 1) << i for i, q in enumerate(pos))
                    got = sum(((g >> q) & 1) << i for i, q in enumerate(pos) if tpos[i] == 255)
                    if op["nruns"] != 255:
                        r = op["runs"]
                        for k in range(0, len(r), 3):
                            got |= ((j >> r[k]) & ((1 << r[k + 1]) - 1)) << r[k + 2]
                    else:
                        got |= sum(((j >> tp) & 1) << i for i, tp in enumerate(tpos) if tp != 255)
                    assert got == want, (pos, tpos, op["runs"], j)
