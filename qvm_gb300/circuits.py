"""Seeded synthetic workloads (gate lists) for tests and benchmarks.

A gate is ``(matrix, qubits)`` with ``qubits`` a nat-tuple: qubits[0] is the
matrix LSB, i.e. the LAST argument of the Quil application
(src/utilities.lisp:43-51).  ``app(name, params, *quil_args)`` converts a
Quil-order application.
"""
from __future__ import annotations

import numpy as np

from .gates import gate_matrix, haar_special_unitary


def app(name, params, *args):
    return gate_matrix(name, *params), [int(a) for a in reversed(args)]


def random_layers(n: int, layers: int = 10, seed: int = 1):
    """20-qubit RX/RZ + CNOT layer circuit: H on all qubits, then per layer
    RX(theta_q), RZ(phi_q) on every qubit (uniform in [0, 2pi)) followed by
    CNOT on pairs (i, i+1) starting at an offset that alternates 0/1."""
    rng = np.random.default_rng(seed)
    gates = [app("H", (), q) for q in range(n)]
    for layer in range(layers):
        th = rng.uniform(0, 2 * np.pi, n)
        ph = rng.uniform(0, 2 * np.pi, n)
        for q in range(n):
            gates.append(app("RX", (th[q],), q))
            gates.append(app("RZ", (ph[q],), q))
        for i in range(layer % 2, n - 1, 2):
            gates.append(app("CNOT", (), i, i + 1))
    return gates


def qft(n: int):
    """QFT on n qubits: for q = n-1 .. 0 apply H q, then CPHASE(pi/2^(q-j))
    j q for each j < q, then the SWAP bit reversal."""
    gates = []
    for q in range(n - 1, -1, -1):
        gates.append(app("H", (), q))
        for j in range(q - 1, -1, -1):
            gates.append(app("CPHASE", (np.pi / 2 ** (q - j),), j, q))
    for i in range(n // 2):
        gates.append(app("SWAP", (), i, n - 1 - i))
    return gates


def qft_examples_order(qubits):
    """The QFT circuit of the reference's examples/qft.lisp:23-62 on the
    given qubits (recursive order, then bit reversal)."""
    qubits = list(qubits)

    def rec(qs):
        q, rest = qs[0], qs[1:]
        if not rest:
            return [app("H", (), q)]
        n = len(rest) + 1
        cr = []
        for i, qi in zip(range(n - 1, 0, -1), rest):
            cr.insert(0, app("CPHASE", (np.pi / 2 ** (n - i),), q, qi))
        return rec(rest) + cr + [app("H", (), q)]

    gates = rec(qubits)
    n = len(qubits)
    for i in range(n // 2):
        gates.append(app("SWAP", (), qubits[i], qubits[n - 1 - i]))
    return gates


def random_su_circuit(n: int, depth: int = 20, seed: int = 3):
    """Per layer: a Haar-random SU(2) on every qubit, then a Haar-random
    SU(4) on each pair of a random perfect matching of the qubits."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(depth):
        for q in range(n):
            gates.append((haar_special_unitary(rng, 2), [q]))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            a, b = int(perm[i]), int(perm[i + 1])
            gates.append((haar_special_unitary(rng, 4), [b, a]))
    return gates


def random_state(n: int, seed: int = 2) -> np.ndarray:
    """Normalised vector of i.i.d. complex Gaussian amplitudes."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v /= np.linalg.norm(v)
    return v.astype(np.complex128)


def random_3_regular_graph(n: int, rng: np.random.Generator, tries: int = 1000):
    """Random simple 3-regular graph on n (even) vertices by the pairing
    model with rejection of loops and multi-edges."""
    if n % 2 or n < 4:
        raise ValueError("a 3-regular graph needs an even n >= 4")
    for _ in range(tries):
        stubs = np.repeat(np.arange(n), 3)
        rng.shuffle(stubs)
        edges = set()
        ok = True
        for i in range(0, len(stubs), 2):
            a, b = int(stubs[i]), int(stubs[i + 1])
            if a == b:
                ok = False
                break
            e = (min(a, b), max(a, b))
            if e in edges:
                ok = False
                break
            edges.add(e)
        if ok:
            return sorted(edges)
    raise RuntimeError("could not sample a 3-regular graph")


def qaoa_maxcut(n: int, edges, gammas, betas):
    """QAOA MaxCut: H on all qubits, then per layer ZZ(gamma) = RZZ(gamma) on
    every edge and RX(2 beta) on every qubit."""
    gates = [app("H", (), q) for q in range(n)]
    for g, b in zip(gammas, betas):
        for (u, v) in edges:
            gates.append(app("RZZ", (g,), u, v))
        for q in range(n):
            gates.append(app("RX", (2 * b,), q))
    return gates


def maxcut_values(n: int, edges) -> np.ndarray:
    """Cut value C(x) = sum over edges of [x_u != x_v] for every basis x."""
    idx = np.arange(1 << n, dtype=np.int64)
    c = np.zeros(1 << n, dtype=np.float64)
    for (u, v) in edges:
        c += ((idx >> u) ^ (idx >> v)) & 1
    return c
