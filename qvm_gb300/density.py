"""Density-matrix QVM: rho of n qubits held as the 2n-qubit vector vec(rho).

Mirrors src/density-qvm.lisp (``density-qvm``, ``make-density-qvm``,
``set-noisy-gate``, ``set-readout-povm``, measurement with readout noise),
the density-matrix methods of src/apply-gate.lisp:42-99,196-209 and
src/measurement.lisp:43-68,77-85,111-122,145-150,
and src/state-representation.lisp:173-290 (row-major vec(rho)).

vec(A rho B) = (A (x) B^T) vec(rho) with row-major vec (the identity of
src/apply-gate.lisp:54-59): row index bits are the high n qubits of the
vector, column bits the low n.  So every operation is an ordinary op of the
2n-qubit statevector engine, and runs through the same fused tile passes:
- a gate U on qubits Q: conj(U) on Q and U on Q + n (two k-qubit ops);
- a noisy gate {K_j}: the superoperator S = sum_j K_j (x) conj(K_j), one
  dense 2k-qubit op on (Q, Q + n).  The reference applies each K_j to a
  pristine copy and accumulates the sum;
- measurement collapse of qubit q: a 2-qubit diagonal on (q, q + n) that
  zeroes the annihilated rows and columns and scales the rest by 1/p;
- MEASURE without an address (dephasing, src/measurement.lisp:111-122):
  the diagonal (1, 0, 0, 1) on (q, q + n).
Outcome probabilities come from the diagonal (``qvmg_density_diagonal``).
"""
from __future__ import annotations

import random

import numpy as np

from . import quil as Q
from .noisy import check_kraus_ops, check_povm, perturb_measurement
from .state import CudaPureState, Program


def gate_ops(matrix, nat_qubits, n: int, perm=None):
    """Ops of U rho U^H on vec(rho): [(kind, data, qubits)]."""
    ghost = [q + n for q in nat_qubits]
    if perm is not None:
        return [("perm", perm, list(nat_qubits)), ("perm", perm, ghost)]
    m = np.asarray(matrix, dtype=np.complex128)
    return [("dense", m.conj(), list(nat_qubits)), ("dense", m, ghost)]


def superoperator(kraus_ops) -> np.ndarray:
    """sum_j K_j (x) conj(K_j): vec(sum_j K_j rho K_j^H) = S vec(rho)."""
    return sum(np.kron(k, np.conj(k)) for k in
               (np.asarray(k, dtype=np.complex128) for k in kraus_ops))


def kraus_ops_on_density(kraus_ops, nat_qubits, n: int):
    """One dense op of 2k qubits: column qubits are the low matrix bits
    (the conj(K) factor), row qubits Q + n the high ones."""
    return [("dense", superoperator(kraus_ops), list(nat_qubits) + [q + n for q in nat_qubits])]


def collapse_diagonal(bit: int, p1: float):
    """force-measurement on rho (src/measurement.lisp:43-68): the diagonal
    over (q, q + n) keeping rows and columns with qubit q = bit, scaled by
    1/P(bit)."""
    if bit == 1:
        return [0.0, 0.0, 0.0, 1.0 / p1]
    return [1.0 / (1.0 - p1), 0.0, 0.0, 0.0]


DEPHASE = [1.0, 0.0, 0.0, 1.0]


class DensityQVM:
    """make-density-qvm: an n-qubit density-matrix simulator on the GPU."""

    def __init__(self, num_qubits: int, precision="fp64", seed: int | None = None,
                 fused: bool = False, fusion_width: int = 2, tile_qubits: int = 0,
                 noisy_gate_definitions=None, readout_povms=None):
        self.num_qubits = int(num_qubits)
        self.state = CudaPureState(2 * self.num_qubits, precision)
        self.rng = random.Random(seed)
        self.fused = fused
        self.fusion_width = fusion_width
        self.tile_qubits = tile_qubits
        self.noisy_gate_definitions = {}
        self.readout_povms = {}
        for (name, qubits), ops in (noisy_gate_definitions or {}).items():
            self.set_noisy_gate(name, qubits, ops)
        for q, povm in (readout_povms or {}).items():
            self.set_readout_povm(q, povm)
        self.program = None
        self.memory = {}
        self._segments = None

    # -- configuration -------------------------------------------------------------
    def set_noisy_gate(self, gate_name: str, qubits, kraus_ops):
        check_kraus_ops(kraus_ops)
        if len(kraus_ops[0]) not in (2, 4):
            raise ValueError("noisy gates act on 1 or 2 qubits")
        self.noisy_gate_definitions[(gate_name, tuple(qubits))] = [
            np.asarray(k, dtype=np.complex128) for k in kraus_ops]
        self._segments = None

    def set_readout_povm(self, qubit: int, povm):
        check_povm(povm)
        self.readout_povms[int(qubit)] = tuple(float(x) for x in povm)

    # -- program -------------------------------------------------------------------------
    def load_program(self, program):
        if isinstance(program, str):
            program = Q.parse(program)
        if program.qubits_needed() > self.num_qubits:
            raise ValueError(f"program needs {program.qubits_needed()} qubits; the QVM has "
                             f"{self.num_qubits}")
        self.program = program
        self.memory = {name: [0] * n for name, n in program.memory.items()}
        self._segments = None
        return self

    def _ops_of(self, ins):
        n = self.num_qubits
        kraus = self.noisy_gate_definitions.get((ins.name, tuple(ins.args)))
        if kraus is not None:
            return kraus_ops_on_density(kraus, ins.qubits, n)
        if ins.kind == "perm":
            return gate_ops(None, ins.qubits, n, perm=ins.perm)
        return gate_ops(ins.matrix, ins.qubits, n)

    def _program(self, apps):
        p = Program()
        for ins in apps:
            for kind, data, qs in self._ops_of(ins):
                if kind == "perm":
                    p.add_permutation(data, qs)
                else:
                    p.add_dense(data, qs)
        if self.fused:
            p.plan(2 * self.num_qubits, self.state.precision, fused=True,
                   fusion_width=self.fusion_width, tile_qubits=self.tile_qubits)
        return p

    def _build(self):
        segs, run = [], []
        for ins in self.program.instructions:
            if isinstance(ins, Q.GateApp):
                run.append(ins)
                continue
            if run:
                segs.append(self._program(run))
                run = []
            segs.append(ins)
        if run:
            segs.append(self._program(run))
        self._segments = segs

    def run(self):
        if self._segments is None:
            self._build()
        for seg in self._segments:
            if isinstance(seg, Program):
                seg.run(self.state, fused=self.fused)
            elif isinstance(seg, Q.Measure):
                if seg.mref is None:
                    self.state.apply_diagonal(DEPHASE, [seg.qubit, seg.qubit + self.num_qubits])
                    continue
                _, bit = self.measure(seg.qubit)
                povm = self.readout_povms.get(seg.qubit)
                if povm is not None:
                    bit = perturb_measurement(bit, povm, self.rng.random())
                self.memory[seg.mref[0]][seg.mref[1]] = bit
            elif isinstance(seg, Q.Reset):
                self.reset_quantum_state()
        return self

    # -- measurement ---------------------------------------------------------------------
    def probabilities(self) -> np.ndarray:
        """density-qvm-measurement-probabilities: Re rho[i][i]."""
        return self.state.density_diagonal()

    def excited_probability(self, q: int) -> float:
        """get-excited-state-probability on rho: the diagonal over bit q = 1."""
        d = self.probabilities()
        idx = np.arange(len(d))
        return float(np.sum(d[(idx >> q) & 1 == 1]))

    def force_measurement(self, bit: int, q: int, excited_probability: float):
        self.state.apply_diagonal(collapse_diagonal(bit, excited_probability),
                                  [q, q + self.num_qubits])

    def measure(self, q: int):
        """measure (src/measurement.lisp:87-105) on rho: (qvm, bit)."""
        if not 0 <= q < self.num_qubits:
            raise ValueError(f"Trying to measure qubit {q} on a QVM with only "
                             f"{self.num_qubits} qubits.")
        p1 = self.excited_probability(q)
        bit = 0 if p1 == 0 else (1 if self.rng.random() <= p1 else 0)
        self.force_measurement(bit, q, p1)
        return self, bit

    def measure_all(self):
        """naive-measure-all (qubits n-1 .. 0, one measure each) plus readout
        noise: the conditional probabilities come from one read of the
        diagonal, and rho becomes |b><b|."""
        n = self.num_qubits
        d = self.probabilities()
        idx = np.arange(len(d))
        mask = np.ones(len(d), dtype=bool)
        bits = [0] * n
        for q in range(n - 1, -1, -1):
            total = float(np.sum(d[mask]))
            p1 = float(np.sum(d[mask & ((idx >> q) & 1 == 1)])) / total
            bit = 0 if p1 == 0 else (1 if self.rng.random() <= p1 else 0)
            bits[q] = bit
            mask &= ((idx >> q) & 1) == bit
        b = sum(bit << q for q, bit in enumerate(bits))
        self.state.set_to_zero_state()
        if b:
            p = Program()
            for q in range(n):
                if (b >> q) & 1:
                    p.add_permutation([1, 0], [q])
                    p.add_permutation([1, 0], [q + n])
            p.run(self.state, fused=False)
            p.free()
        out = []
        for q, bit in enumerate(bits):
            povm = self.readout_povms.get(q)
            out.append(perturb_measurement(bit, povm, self.rng.random()) if povm else bit)
        return self, out

    # -- state access --------------------------------------------------------------------
    def matrix_view(self) -> np.ndarray:
        """rho as a 2^n x 2^n complex128 matrix (downloaded)."""
        dim = 1 << self.num_qubits
        return self.state.state_elements().reshape(dim, dim)

    def set_density_matrix(self, rho):
        rho = np.asarray(rho, dtype=np.complex128)
        dim = 1 << self.num_qubits
        if rho.shape != (dim, dim):
            raise ValueError(f"expected a {dim} x {dim} density matrix")
        self.state.set_state_elements(rho.reshape(-1))

    def reset_quantum_state(self):
        self.state.set_to_zero_state()

    def reset_classical_memory(self):
        self.memory = {k: [0] * len(v) for k, v in self.memory.items()}

    def memory_ref(self, name: str, index: int = 0) -> int:
        return self.memory[name][index]

    def free(self):
        self.state.free()


def make_density_qvm(num_qubits: int, **kw) -> DensityQVM:
    return DensityQVM(num_qubits, **kw)
