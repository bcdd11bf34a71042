"""Standard Quil gate matrices (quil/stdgates.quil), complex128, row-major.

The reference obtains these from cl-quil's ``gate-matrix``
(src/apply-gate.lisp:109-160); the textual definitions it ships are
quil/stdgates.quil, restated here.  ``cis(x)`` is exp(i x).
"""
from __future__ import annotations

import numpy as np


def _cis(x):
    return np.cos(x) + 1j * np.sin(x)


def _m(rows):
    return np.array(rows, dtype=np.complex128)


_R2 = 1.0 / np.sqrt(2.0)


def _rx(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return _m([[c, -1j * s], [-1j * s, c]])


def _ry(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return _m([[c, -s], [s, c]])


def _rz(t):
    return _m([[_cis(-t / 2), 0], [0, _cis(t / 2)]])


def _cphase(slot):
    def f(a):
        m = np.eye(4, dtype=np.complex128)
        m[slot, slot] = _cis(a)
        return m
    return f


def _rzz(p):
    return np.diag([_cis(-p / 2), _cis(p / 2), _cis(p / 2), _cis(-p / 2)]).astype(np.complex128)


def _rxx(p):
    c, s = np.cos(p / 2), np.sin(p / 2)
    return _m([[c, 0, 0, -1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [-1j * s, 0, 0, c]])


def _ryy(p):
    c, s = np.cos(p / 2), np.sin(p / 2)
    return _m([[c, 0, 0, 1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [1j * s, 0, 0, c]])


def _piswap(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return _m([[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, 1]])


def _pswap(t):
    return _m([[1, 0, 0, 0], [0, 0, _cis(t), 0], [0, _cis(t), 0, 0], [0, 0, 0, 1]])


def _fsim(t, p):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return _m([[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, _cis(p)]])


def _ccnot():
    m = np.eye(8, dtype=np.complex128)
    m[6, 6] = m[7, 7] = 0
    m[6, 7] = m[7, 6] = 1
    return m


def _cswap():
    m = np.eye(8, dtype=np.complex128)
    m[5, 5] = m[6, 6] = 0
    m[5, 6] = m[6, 5] = 1
    return m


STANDARD_GATES = {
    # name: (number of parameters, constructor)
    "I": (0, lambda: np.eye(2, dtype=np.complex128)),
    "X": (0, lambda: _m([[0, 1], [1, 0]])),
    "Y": (0, lambda: _m([[0, -1j], [1j, 0]])),
    "Z": (0, lambda: _m([[1, 0], [0, -1]])),
    "H": (0, lambda: _m([[_R2, _R2], [_R2, -_R2]])),
    "RX": (1, _rx),
    "RY": (1, _ry),
    "RZ": (1, _rz),
    "S": (0, lambda: _m([[1, 0], [0, 1j]])),
    "T": (0, lambda: _m([[1, 0], [0, _cis(np.pi / 4)]])),
    "PHASE": (1, lambda a: _m([[1, 0], [0, _cis(a)]])),
    "CNOT": (0, lambda: _m([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])),
    "CZ": (0, lambda: np.diag([1, 1, 1, -1]).astype(np.complex128)),
    "CPHASE00": (1, _cphase(0)),
    "CPHASE01": (1, _cphase(1)),
    "CPHASE10": (1, _cphase(2)),
    "CPHASE": (1, _cphase(3)),
    "SWAP": (0, lambda: _m([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]])),
    "ISWAP": (0, lambda: _m([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]])),
    "SQISWAP": (0, lambda: _m([[1, 0, 0, 0], [0, _R2, 1j * _R2, 0], [0, 1j * _R2, _R2, 0],
                               [0, 0, 0, 1]])),
    "PSWAP": (1, _pswap),
    "RZZ": (1, _rzz),
    "RXX": (1, _rxx),
    "RYY": (1, _ryy),
    "PISWAP": (1, _piswap),
    "XY": (1, _piswap),
    "FSIM": (2, _fsim),
    "CCNOT": (0, _ccnot),
    "CSWAP": (0, _cswap),
}


def gate_matrix(name: str, *params) -> np.ndarray:
    """Matrix of a standard gate with its parameters."""
    try:
        nparams, ctor = STANDARD_GATES[name]
    except KeyError:
        raise KeyError(f"unknown gate {name}") from None
    if len(params) != nparams:
        raise ValueError(f"gate {name} takes {nparams} parameters, got {len(params)}")
    return ctor(*[float(p) for p in params])


def controlled(m: np.ndarray) -> np.ndarray:
    """CONTROLLED modifier: block diag(I, M), control = new matrix MSB."""
    d = m.shape[0]
    out = np.eye(2 * d, dtype=np.complex128)
    out[d:, d:] = m
    return out


def dagger(m: np.ndarray) -> np.ndarray:
    """DAGGER modifier: conjugate transpose."""
    return np.conj(m).T.copy()


def permutation_matrix(perm) -> np.ndarray:
    """Matrix of a permutation gate, new amplitude j = old amplitude perm[j]
    (the transposition semantics of src/compile-gate.lisp:259-279)."""
    d = len(perm)
    m = np.zeros((d, d), dtype=np.complex128)
    for j, p in enumerate(perm):
        m[j, p] = 1
    return m


def haar_unitary(rng: np.random.Generator, d: int) -> np.ndarray:
    """Haar-random d x d unitary (QR of a complex Gaussian matrix with the
    phases of R's diagonal divided out, Mezzadri's construction)."""
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return (q * ph).astype(np.complex128)


def haar_special_unitary(rng: np.random.Generator, d: int) -> np.ndarray:
    u = haar_unitary(rng, d)
    det = np.linalg.det(u)
    return (u / det ** (1.0 / d)).astype(np.complex128)
