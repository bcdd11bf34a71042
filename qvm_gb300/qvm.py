"""``PureStateQVM``: the reference's pure-state QVM API over the GPU state.

Mirrors src/qvm.lisp (make-qvm :150-164, load-program, reset-quantum-state
:84-87), src/execution.lisp (run :31-37), src/transition.lisp (gate
applications :155-186, MEASURE :119-135, RESET), src/measurement.lisp
(measure :87-105, measure-all :122-143) and src/compile-gate.lisp (measure
chains and the compiled measurement convention).  Random draws come from a
host MT19937 stream (``random.Random``) in the reference's order, and are
passed to the device, so a run is reproducible from its seed.

Consecutive gate applications between classical instructions are handed to
the device as one ``Program`` and run in plain (one pass per gate) or fused
mode; measurements run on the device with the host's draw.
"""
from __future__ import annotations

import random

import numpy as np

from . import quil as Q
from .state import CudaPureState, Program


class PureStateQVM:
    def __init__(self, num_qubits: int, precision="fp64", seed: int | None = None,
                 compile: bool = False, fused: bool = False, fusion_width: int = 2,
                 tile_qubits: int = 0):
        self.num_qubits = int(num_qubits)
        self.state = CudaPureState(self.num_qubits, precision)
        self.rng = random.Random(seed)
        self.compile = compile
        self.fused = fused
        self.fusion_width = fusion_width
        self.tile_qubits = tile_qubits
        self.memory: dict[str, list[int]] = {}
        self.program: Q.Program | None = None
        self._segments = []

    # -- make-qvm / load-program ------------------------------------------------
    def load_program(self, program):
        if isinstance(program, str):
            program = Q.parse(program)
        if program.qubits_needed() > self.num_qubits:
            raise ValueError(f"program needs {program.qubits_needed()} qubits; the QVM has "
                             f"{self.num_qubits}")
        self.program = program
        self.memory = {name: [0] * n for name, n in program.memory.items()}
        instrs = program.instructions
        if self.compile:
            instrs = Q.compile_measure_chains(instrs, self.num_qubits)
        # Group consecutive gate applications into device programs.
        self._segments = []
        run = []
        for ins in instrs:
            if isinstance(ins, Q.GateApp):
                run.append(ins)
                continue
            if run:
                self._segments.append(self._make_program(run))
                run = []
            self._segments.append(ins)
        if run:
            self._segments.append(self._make_program(run))
        return self

    def _make_program(self, apps):
        p = Program()
        for a in apps:
            if a.kind == "perm":
                p.add_permutation(a.perm, a.qubits)
            else:
                p.add_dense(a.matrix, a.qubits)
        if self.fused:
            p.plan(self.num_qubits, self.state.precision, fused=True,
                   fusion_width=self.fusion_width, tile_qubits=self.tile_qubits)
        return p

    # -- run ----------------------------------------------------------------------
    def run(self):
        for seg in self._segments:
            if isinstance(seg, Program):
                seg.run(self.state, fused=self.fused)
            elif isinstance(seg, Q.Measure):
                _, bit = self.measure(seg.qubit)
                if seg.mref is not None:
                    self.memory[seg.mref[0]][seg.mref[1]] = bit
            elif isinstance(seg, Q.MeasureAll):
                _, bits = self.measure_all()
                for q, (name, idx) in seg.storage:
                    self.memory[name][idx] = bits[q]
            elif isinstance(seg, Q.Reset):
                self.state.set_to_zero_state()
        return self

    # -- measurement ----------------------------------------------------------------
    def measure(self, q: int):
        """(qvm, bit): the interpreted convention by default, the compiled
        one when the QVM compiles its program."""
        if not 0 <= q < self.num_qubits:
            raise ValueError(f"Trying to measure qubit {q} on a QVM with only "
                             f"{self.num_qubits} qubits.")
        if self.compile:
            draw = self.rng.random()
            bit, _, _ = self.state.measure(q, draw, compiled=True)
        else:
            # The interpreted measure draws only when p1 != 0; the device
            # reports whether it used the draw, and an unused draw is
            # returned to the stream by rewinding it.
            saved = self.rng.getstate()
            draw = self.rng.random()
            bit, used, _ = self.state.measure(q, draw, compiled=False)
            if not used:
                self.rng.setstate(saved)
        return self, bit

    def measure_all(self):
        """(qvm, bits LSB-first) (src/measurement.lisp:128-143)."""
        idx = self.state.measure_all(self.rng.random())
        return self, [(idx >> i) & 1 for i in range(self.num_qubits)]

    # -- state access -------------------------------------------------------------------
    @property
    def amplitudes(self) -> np.ndarray:
        return self.state.state_elements()

    def probabilities(self) -> np.ndarray:
        return self.state.probabilities()

    def reset_quantum_state(self):
        self.state.set_to_zero_state()

    def reset_classical_memory(self):
        self.memory = {k: [0] * len(v) for k, v in self.memory.items()}

    def memory_ref(self, name: str, index: int = 0) -> int:
        return self.memory[name][index]

    def free(self):
        self.state.free()


def make_qvm(num_qubits: int, **kw) -> PureStateQVM:
    return PureStateQVM(num_qubits, **kw)


def run_program(num_qubits: int, program, **kw) -> PureStateQVM:
    """run-program: make a QVM, load the program, run it."""
    q = PureStateQVM(num_qubits, **kw)
    q.load_program(program)
    return q.run()
