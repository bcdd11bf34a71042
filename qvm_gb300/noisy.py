"""Noisy pure-state QVMs: stochastic Kraus maps, readout POVMs, depolarizing noise.

Mirrors src/noisy-qvm.lisp (``noisy-qvm``: noisy gate definitions as Kraus
maps, readout POVMs), src/channel-qvm.lisp:109-205 (``check-kraus-ops``,
``perturb-measurement``, ``check-povm``), src/measurement.lisp:228-244
(``perturb-measured-bits``) and src/depolarizing-noise.lisp
(``depolarizing-qvm``).

A noisy gate is one device call, ``qvmg_apply_kraus``: one reduction of the
gate qubits' reduced density matrix gives every ||K_j psi||^2, and the
chosen K_j / sqrt(p_j) is applied in one pass (src/apply-gate.lisp:16-39
copies the state and applies operators one by one instead).  Gates without a
noisy definition run as device programs, as in ``PureStateQVM``.  The
depolarizing QVM's Pauli errors do not depend on the state, so a run's
errors are drawn on the host in the reference's order and inserted into the
gate program as permutation and diagonal ops.
"""
from __future__ import annotations

import numpy as np

from . import quil as Q
from .gates import gate_matrix
from .qvm import PureStateQVM
from .state import Program


# ---- Kraus maps and POVMs (src/noisy-qvm.lisp:46-82, src/channel-qvm.lisp) -------------

def make_pauli_noise_map(px: float, py: float, pz: float):
    """Kraus operators of rho -> (1-px-py-pz) rho + px X rho X + py Y rho Y + pz Z rho Z:
    [sqrt(1-sum) I (when sum < 1), sqrt(px) X, sqrt(py) Y, sqrt(pz) Z]."""
    for p in (px, py, pz):
        if not 0 <= p <= 1:
            raise ValueError("Pauli noise probabilities lie in [0, 1]")
    psum = px + py + pz
    if not 0 <= psum <= 1:
        raise ValueError("Pauli noise probabilities sum to at most 1")
    ops = [np.sqrt(p) * gate_matrix(s) for s, p in (("X", px), ("Y", py), ("Z", pz))]
    if psum < 1:
        ops.insert(0, np.sqrt(1.0 - psum) * np.eye(2, dtype=np.complex128))
    return ops


def make_pauli_perturbed_1q_gate(gate_name: str, px: float, py: float, pz: float):
    """The standard gate U followed by the Pauli noise map: [K_j U]."""
    u = gate_matrix(gate_name)
    return [k @ u for k in make_pauli_noise_map(px, py, pz)]


def check_kraus_ops(kraus_ops, tol: float = 1e-5):
    """Square, equal-sized operators with sum K^H K = I (within tol)."""
    if not kraus_ops:
        raise ValueError("empty Kraus map")
    m = np.asarray(kraus_ops[0]).shape[0]
    acc = np.zeros((m, m), dtype=np.complex128)
    for k in kraus_ops:
        k = np.asarray(k, dtype=np.complex128)
        if k.shape != (m, m):
            raise ValueError("All Kraus operators must have matching dimensions")
        acc += k.conj().T @ k
    if not np.allclose(acc, np.eye(m), atol=tol, rtol=0):
        raise ValueError("The Kraus map must preserve trace: sum K^H K must be the identity")


def check_povm(povm):
    """(p(0|0), p(0|1), p(1|0), p(1|1)) with both columns summing to 1."""
    p00, p01, p10, p11 = (float(x) for x in povm)
    for p in (p00, p01, p10, p11):
        if not 0.0 <= p <= 1.0:
            raise ValueError("POVM entries lie in [0, 1]")
    if abs(p00 + p10 - 1.0) > 1e-10 or abs(p01 + p11 - 1.0) > 1e-10:
        raise ValueError("POVM columns must sum to 1")


def perturb_measurement(actual: int, povm, draw: float) -> int:
    """perturb-measurement (src/channel-qvm.lisp:185-195)."""
    p00, p01, _, _ = povm
    if actual == 0:
        return 0 if draw <= p00 else 1
    return 0 if draw <= p01 else 1


# ---- noisy-qvm --------------------------------------------------------------------------

class _Kraus:
    def __init__(self, ops, qubits):
        self.ops = ops
        self.qubits = qubits


class NoisyQVM(PureStateQVM):
    """A pure-state QVM with noisy gate definitions and readout POVMs."""

    def __init__(self, num_qubits: int, noisy_gate_definitions=None, readout_povms=None, **kw):
        kw.pop("compile", None)  # the noisy QVM does not compile its program
        super().__init__(num_qubits, compile=False, **kw)
        self.noisy_gate_definitions = {}
        self.readout_povms = {}
        for (name, qubits), ops in (noisy_gate_definitions or {}).items():
            self.set_noisy_gate(name, qubits, ops)
        for q, povm in (readout_povms or {}).items():
            self.set_readout_povm(q, povm)
        self._built_for = None

    def set_noisy_gate(self, gate_name: str, qubits, kraus_ops):
        check_kraus_ops(kraus_ops)
        if len(kraus_ops[0]) not in (2, 4):
            raise ValueError("noisy gates act on 1 or 2 qubits")
        self.noisy_gate_definitions[(gate_name, tuple(qubits))] = [
            np.asarray(k, dtype=np.complex128) for k in kraus_ops]
        self._built_for = None

    def set_readout_povm(self, qubit: int, povm):
        check_povm(povm)
        self.readout_povms[int(qubit)] = tuple(float(x) for x in povm)

    def load_program(self, program):
        if isinstance(program, str):
            program = Q.parse(program)
        super().load_program(program)
        self._built_for = None
        return self

    def _build(self):
        """Segments with noisy gate applications split out as Kraus steps."""
        segs, run = [], []
        for ins in self.program.instructions:
            if isinstance(ins, Q.GateApp):
                ops = self.noisy_gate_definitions.get((ins.name, tuple(ins.args)))
                if ops is None:
                    run.append(ins)
                    continue
                if run:
                    segs.append(self._make_program(run))
                    run = []
                segs.append(_Kraus(ops, ins.qubits))
                continue
            if run:
                segs.append(self._make_program(run))
                run = []
            segs.append(ins)
        if run:
            segs.append(self._make_program(run))
        self._segments = segs
        self._built_for = len(self.noisy_gate_definitions)

    def run(self):
        if self._built_for != len(self.noisy_gate_definitions):
            self._build()
        for seg in self._segments:
            if isinstance(seg, _Kraus):
                self.state.apply_kraus(seg.ops, seg.qubits, self.rng.random())
            elif isinstance(seg, Program):
                seg.run(self.state, fused=self.fused)
            elif isinstance(seg, Q.Measure):
                _, bit = self.measure(seg.qubit)
                if seg.mref is not None:
                    povm = self.readout_povms.get(seg.qubit)
                    if povm is not None:
                        bit = perturb_measurement(bit, povm, self.rng.random())
                    self.memory[seg.mref[0]][seg.mref[1]] = bit
            elif isinstance(seg, Q.Reset):
                self.state.set_to_zero_state()
        return self

    def measure_all(self):
        """measure-all with the readout POVMs applied to the bits
        (src/measurement.lisp:228-244)."""
        qvm, bits = super().measure_all()
        out = []
        for q, b in enumerate(bits):
            povm = self.readout_povms.get(q)
            out.append(perturb_measurement(b, povm, self.rng.random()) if povm else b)
        return qvm, out


# ---- depolarizing-qvm -------------------------------------------------------------------

class DepolarizingQVM(PureStateQVM):
    """Pauli errors with probabilities (x, y, z) on every qubit a gate
    touches (after the gate) and on every qubit after a RESET, and with
    (measure_x, measure_y, measure_z) on a qubit before it is measured."""

    def __init__(self, num_qubits: int, x=0.0, y=0.0, z=0.0, measure_x=0.0, measure_y=0.0,
                 measure_z=0.0, **kw):
        kw.pop("compile", None)
        super().__init__(num_qubits, compile=False, **kw)
        self.gate_noise = (float(x), float(y), float(z))
        self.measure_noise = (float(measure_x), float(measure_y), float(measure_z))
        for p in self.gate_noise + self.measure_noise:
            if not 0 <= p <= 1:
                raise ValueError("noise probabilities lie in [0, 1]")
        if sum(self.gate_noise) > 1 or sum(self.measure_noise) > 1:
            raise ValueError("noise probabilities sum to at most 1")

    def _noise(self, px, py, pz):
        """add-depolarizing-noise's choice (src/depolarizing-noise.lisp:42-70):
        None, "X", "Y" or "Z"; one draw, plus one more when an error occurs."""
        total = px + py + pz
        if not self.rng.random() < total:
            return None
        px, py, pz = px / total, py / total, pz / total
        r = self.rng.random()
        if r < px:
            return "X"
        r -= px
        if r < py:
            return "Y"
        r -= py
        if r < pz:
            return "Z"
        return None

    @staticmethod
    def _add_pauli(prog: Program, pauli: str, q: int):
        if pauli == "X":
            prog.add_permutation([1, 0], [q])
        elif pauli == "Z":
            prog.add_diagonal([1.0, -1.0], [q])
        else:
            prog.add_dense(gate_matrix("Y"), [q])

    def run(self):
        prog, pending = Program(), 0

        def flush():
            nonlocal prog, pending
            if pending:
                if self.fused:
                    prog.plan(self.num_qubits, self.state.precision, fused=True,
                              fusion_width=self.fusion_width, tile_qubits=self.tile_qubits)
                prog.run(self.state, fused=self.fused)
                prog.free()
                prog, pending = Program(), 0

        for ins in self.program.instructions:
            if isinstance(ins, Q.GateApp):
                if ins.kind == "perm":
                    prog.add_permutation(ins.perm, ins.qubits)
                else:
                    prog.add_dense(ins.matrix, ins.qubits)
                pending += 1
                for q in ins.args:
                    e = self._noise(*self.gate_noise)
                    if e:
                        self._add_pauli(prog, e, q)
                continue
            if isinstance(ins, Q.Measure):
                e = self._noise(*self.measure_noise)
                if e:
                    self._add_pauli(prog, e, ins.qubit)
                    pending += 1
                flush()
                _, bit = self.measure(ins.qubit)
                if ins.mref is not None:
                    self.memory[ins.mref[0]][ins.mref[1]] = bit
            elif isinstance(ins, Q.Reset):
                flush()
                self.state.set_to_zero_state()
                for q in range(self.num_qubits):
                    e = self._noise(*self.gate_noise)
                    if e:
                        self._add_pauli(prog, e, q)
                        pending += 1
        flush()
        prog.free()
        return self
