"""The QVM server's pure-state endpoints over a device-resident state.

Mirrors app/src/api of the reference:
- ``perform_multishot`` (app/src/api/multishot.lisp:52-101): run a program
  ``num_trials`` times and return the requested classical memory per trial;
- ``perform_multishot_measure`` (app/src/api/multishot-measure.lisp:7-109):
  run a program once and measure a list of qubits on ``num_trials`` reloads
  of the prepared state;
- ``perform_expectation`` (app/src/api/expectation.lisp:27-89): <F|O|F> for
  each operator program O on the prepared state F;
- ``perform_wavefunction`` / ``perform_probabilities`` with the wire
  formats of app/src/handle-request.lisp:132-175 (big-endian doubles,
  app/src/utilities.lisp:40-87).

The reference re-runs the program (multishot) or copies the prepared state
back (multishot-measure, expectation) once per trial or operator.  Here the
prepared state stays in HBM:
- trials whose measurements all come after the last gate are replayed from
  the marginal distribution of the measured qubits, which is reduced once
  on the device (``qvmg_measure_sequence``).  Every trial takes the same
  draws, in the same order, with the same skip when p1 = 0, as the
  reference's per-trial ``measure`` calls;
- measuring every qubit is the reference's measure-all fast path: one
  bisection sample per trial (``qvmg_sample``);
- expectation values copy the prepared state device-to-device and take the
  inner product on the device.

Programs with a gate after a measurement, a RESET, or measure chains mixed
with single measurements run trial by trial on the device, as the reference
does.  Draws come from the caller's MT19937 stream (``random.Random``), and
an unused draw is returned to it.
"""
from __future__ import annotations

import random

from . import _lib as L
from . import quil as Q
from .qvm import PureStateQVM
from .state import CudaPureState, Program


def _as_program(quil):
    return Q.parse(quil) if isinstance(quil, str) else quil


def _take_draws(rng: random.Random, count: int):
    """Draw ``count`` numbers; returns (draws, rewind) where rewind(used)
    puts the stream right after the first ``used`` draws."""
    saved = rng.getstate()
    draws = [rng.random() for _ in range(count)]

    def rewind(used: int):
        rng.setstate(saved)
        for _ in range(used):
            rng.random()

    return draws, rewind


# ---- wavefunction / probabilities -------------------------------------------------

def perform_wavefunction(quil, num_qubits: int, **qvm_kw) -> PureStateQVM:
    """Run the program; the state stays on the device (perform-wavefunction)."""
    qvm = PureStateQVM(num_qubits, **qvm_kw)
    qvm.load_program(_as_program(quil))
    return qvm.run()


def perform_probabilities(quil, num_qubits: int, **qvm_kw):
    """(qvm, |a_i|^2 for every basis state) (app/src/api/probabilities.lisp)."""
    qvm = perform_wavefunction(quil, num_qubits, **qvm_kw)
    return qvm, qvm.state.probabilities()


def wavefunction_octets(qvm_or_state) -> memoryview:
    """The wavefunction endpoint's reply body: 16 octets per amplitude."""
    s = qvm_or_state.state if isinstance(qvm_or_state, PureStateQVM) else qvm_or_state
    return s.wavefunction_octets()


def probabilities_octets(qvm_or_state) -> memoryview:
    """The probabilities endpoint's reply body: 8 octets per probability."""
    s = qvm_or_state.state if isinstance(qvm_or_state, PureStateQVM) else qvm_or_state
    return s.probabilities_octets()


# ---- multishot-measure ----------------------------------------------------------------

UNUSED = -1  # the reference's :unused-qubit


def relabel(qubits, num_qubits: int, relabeling):
    """Qubit relabeling of %perform-multishot-measure: a qubit becomes its
    position in ``relabeling`` (UNUSED when absent); the qubit count grows
    to cover the used positions."""
    if relabeling is None:
        return list(qubits), num_qubits
    rl = list(relabeling)
    out = [rl.index(q) if q in rl else UNUSED for q in qubits]
    used = [q for q in out if q != UNUSED]
    return out, max(num_qubits, 1 + max(used, default=-1))


def measure_trials(state: CudaPureState, qubits, num_trials: int, rng: random.Random):
    """parallel-measure on ``num_trials`` reloads of ``state`` (interpreted
    measure): a list of per-trial bit lists."""
    n = state.num_qubits()
    distinct = {q for q in qubits if q != UNUSED}
    if len(distinct) == n:
        # measure-all fast path: one draw per trial, bisection sampling
        draws = [rng.random() for _ in range(num_trials)]
        idx = state.sample(draws, rule="bisect")
        return [[0 if q == UNUSED else int((int(i) >> q) & 1) for q in qubits] for i in idx]
    draws, rewind = _take_draws(rng, num_trials * len(qubits))
    bits, used = state.measure_sequence(qubits, draws, num_trials, compiled=False)
    rewind(used)
    return bits.astype(int).tolist()


def perform_multishot_measure(quil, num_qubits: int, qubits, num_trials: int, relabeling=None,
                              rng: random.Random | None = None, **qvm_kw):
    """Run ``quil`` once, then measure ``qubits`` (in order) on each of
    ``num_trials`` copies of the prepared state."""
    qubits = list(qubits)
    if any((not isinstance(q, int)) or q < 0 for q in qubits):
        raise ValueError("qubits must be non-negative integers")
    if not qubits or num_trials == 0:
        return []
    qubits, num_qubits = relabel(qubits, num_qubits, relabeling)
    if any(q != UNUSED and q >= num_qubits for q in qubits):
        raise ValueError(f"The provided qubits {qubits} to a multishot measure are out of "
                         f"range for the given QVM, which only has {num_qubits} qubits.")
    rng = rng if rng is not None else random.Random()
    qvm = PureStateQVM(num_qubits, **qvm_kw)
    try:
        qvm.load_program(_as_program(quil))
        qvm.run()
        return measure_trials(qvm.state, qubits, num_trials, rng)
    finally:
        qvm.free()


# ---- multishot -----------------------------------------------------------------------------

def valid_address_query(addresses) -> bool:
    """valid-address-query-p (app/src/api/multishot.lisp:17-29)."""
    if not isinstance(addresses, dict):
        return False
    for k, v in addresses.items():
        if not isinstance(k, str):
            return False
        if v is True or v is None:  # None is the empty list (JSON null)
            continue
        if not (isinstance(v, list) and all(isinstance(i, int) and i >= 0 for i in v)):
            return False
    return True


def _collect(memory, addresses, results):
    """collect-result-data (app/src/api/multishot.lisp:31-48)."""
    for name, idx in addresses.items():
        if idx is True:
            results[name].append(list(memory[name]))
        else:
            results[name].append([memory[name][i] for i in (idx or [])])


def _terminal_measurements(segments):
    """(gate programs, measurements) when every measurement follows the last
    gate and nothing else intervenes; None otherwise."""
    gates, meas = [], []
    for seg in segments:
        if isinstance(seg, Program):
            if meas:
                return None
            gates.append(seg)
        elif isinstance(seg, (Q.Measure, Q.MeasureAll)):
            meas.append(seg)
        else:
            return None
    kinds = {type(m) for m in meas}
    if len(kinds) > 1 or (Q.MeasureAll in kinds and len(meas) > 1):
        return None
    return gates, meas


def perform_multishot(quil, num_qubits: int, addresses: dict, num_trials: int,
                      rng: random.Random | None = None, **qvm_kw) -> dict:
    """Run ``quil`` ``num_trials`` times; per requested memory name, the
    list of per-trial values."""
    if not valid_address_query(addresses):
        raise ValueError("Detected invalid address query in multishot experiment.")
    if (not addresses or num_trials == 0
            or all(v is None for v in addresses.values())):
        return {}
    rng = rng if rng is not None else random.Random(qvm_kw.pop("seed", None))
    qvm = PureStateQVM(num_qubits, **qvm_kw)
    qvm.rng = rng
    results = {name: [] for name in addresses}
    try:
        qvm.load_program(_as_program(quil))
        term = _terminal_measurements(qvm._segments)
        if term is None:
            for _ in range(num_trials):
                if num_trials != 1:
                    qvm.reset_quantum_state()
                qvm.run()
                _collect(qvm.memory, addresses, results)
            return results
        gates, meas = term
        for g in gates:
            g.run(qvm.state, fused=qvm.fused)
        if meas and isinstance(meas[0], Q.MeasureAll):
            draws = [rng.random() for _ in range(num_trials)]
            idx = qvm.state.sample(draws, rule="bisect")
            for i in idx:
                for q, (name, k) in meas[0].storage:
                    qvm.memory[name][k] = int((int(i) >> q) & 1)
                _collect(qvm.memory, addresses, results)
            return results
        qubits = [m.qubit for m in meas]
        if qubits:
            draws, rewind = _take_draws(rng, num_trials * len(qubits))
            bits, used = qvm.state.measure_sequence(qubits, draws, num_trials,
                                                    compiled=qvm.compile)
            rewind(used)
        for t in range(num_trials):
            for e, m in enumerate(meas):
                if m.mref is not None:
                    qvm.memory[m.mref[0]][m.mref[1]] = int(bits[t, e])
            _collect(qvm.memory, addresses, results)
        return results
    finally:
        qvm.free()


# ---- expectation ---------------------------------------------------------------------------

def perform_expectation(state_prep, operators, num_qubits: int, **qvm_kw):
    """[<F|O_1|F>, <F|O_2|F>, ...] (real parts) for the state F that
    ``state_prep`` makes from |0...0>.  The imaginary parts must vanish:
    below 1e-14 for FP64 states as in the reference, below 1e-6 for FP32."""
    operators = list(operators)
    if not operators:
        return []
    prep = PureStateQVM(num_qubits, **qvm_kw)
    work = PureStateQVM(num_qubits, **qvm_kw)
    tol = 1e-14 if prep.state.precision == L.FP64 else 1e-6
    try:
        prep.load_program(_as_program(state_prep))
        prep.run()
        out = []
        for op in operators:
            work.state.copy_from(prep.state)
            work.load_program(_as_program(op))
            work.run()
            e = prep.state.inner(work.state)
            if abs(e.imag) >= tol:
                raise ArithmeticError(f"non-vanishing imaginary part of an expectation value: {e}")
            out.append(e.real)
        return out
    finally:
        prep.free()
        work.free()
