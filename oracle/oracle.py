"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference QVM's pure-state
algorithms (``qvm_oracle.c``; each function cites the Lisp file:line it
follows).  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` load it, and only as the checker or the timed CPU
baseline -- the product path (``qvm_gb300``) never imports this module.

Wavefunctions are numpy ``complex128`` vectors of length 2^n, LSB-first.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        sig = {
            "orc_inject_bit": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_int]),
            "orc_eject_bit": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_int]),
            "orc_index_to_address": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]),
            "orc_subdivide": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int, _u64p, _u64p]),
            "orc_set_workers": (None, [ctypes.c_int]),
            "orc_get_workers": (ctypes.c_int, []),
            "orc_set_parallel_threshold": (None, [ctypes.c_int]),
            "orc_bring_to_zero": (None, [_dp, ctypes.c_uint64]),
            "orc_copy": (None, [_dp, _dp, ctypes.c_uint64]),
            "orc_ground_probability": (ctypes.c_double, [_dp, ctypes.c_int, ctypes.c_int]),
            "orc_excited_probability": (ctypes.c_double, [_dp, ctypes.c_int, ctypes.c_int]),
            "orc_norm": (ctypes.c_double, [_dp, ctypes.c_uint64]),
            "orc_normalize": (None, [_dp, ctypes.c_uint64, ctypes.c_double]),
            "orc_apply_matrix_operator": (None, [_dp, ctypes.c_int, _dp, ctypes.c_int, _ip]),
            "orc_apply_permutation": (None, [_dp, ctypes.c_int, ctypes.c_int, _ip, _i64p]),
            "orc_permutation_to_transpositions": (ctypes.c_int, [ctypes.c_int, _i64p, _ip, _ip]),
            "orc_force_measurement": (None, [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
            "orc_measure": (ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _ip, _dp]),
            "orc_measure_compiled": (ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]),
            "orc_sample_bisect": (ctypes.c_uint64, [_dp, ctypes.c_uint64, ctypes.c_double]),
            "orc_measure_all": (ctypes.c_uint64, [_dp, ctypes.c_int, ctypes.c_double]),
            "orc_cdf": (None, [_dp, ctypes.c_uint64, _dp]),
            "orc_sample_multiple": (None, [_dp, ctypes.c_uint64, _dp, ctypes.c_uint64, _u64p]),
            "orc_inner": (None, [_dp, _dp, ctypes.c_uint64, _dp, _dp]),
            "orc_gate_matrix": (ctypes.c_int, [ctypes.c_char_p, _dp, ctypes.c_int, _dp, _ip]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _wf_ptr(wf: np.ndarray):
    assert wf.dtype == np.complex128 and wf.flags["C_CONTIGUOUS"]
    return wf.ctypes.data_as(_dp)


def _qubits(qubits):
    arr = (ctypes.c_int * len(qubits))(*[int(q) for q in qubits])
    return arr


def nqubits_of(wf: np.ndarray) -> int:
    return max(1, int(len(wf)).bit_length() - 1)


# --- utilities ------------------------------------------------------------
def inject_bit(x: int, n: int) -> int:
    return lib().orc_inject_bit(x, n)


def eject_bit(x: int, n: int) -> int:
    return lib().orc_eject_bit(x, n)


def index_to_address(index: int, qubit: int, state: int) -> int:
    return lib().orc_index_to_address(index, qubit, state)


def subdivide(total: int, num_ranges: int):
    s = (ctypes.c_uint64 * max(1, num_ranges))()
    e = (ctypes.c_uint64 * max(1, num_ranges))()
    n = lib().orc_subdivide(total, num_ranges, s, e)
    return [(s[i], e[i]) for i in range(n)]


def set_workers(workers: int, threshold: int | None = None):
    lib().orc_set_workers(int(workers))
    if threshold is not None:
        lib().orc_set_parallel_threshold(int(threshold))


# --- state ----------------------------------------------------------------
def zero_state(nq: int) -> np.ndarray:
    wf = np.zeros(1 << nq, dtype=np.complex128)
    lib().orc_bring_to_zero(_wf_ptr(wf), len(wf))
    return wf


def bring_to_zero(wf: np.ndarray) -> np.ndarray:
    lib().orc_bring_to_zero(_wf_ptr(wf), len(wf))
    return wf


def ground_probability(wf, q):
    return lib().orc_ground_probability(_wf_ptr(wf), nqubits_of(wf), q)


def excited_probability(wf, q):
    return lib().orc_excited_probability(_wf_ptr(wf), nqubits_of(wf), q)


def norm(wf):
    return lib().orc_norm(_wf_ptr(wf), len(wf))


def normalize(wf, length: float = 0.0):
    lib().orc_normalize(_wf_ptr(wf), len(wf), float(length))
    return wf


def apply_matrix_operator(wf, matrix, qubits):
    """Apply ``matrix`` (2^k x 2^k) on the nat-tuple ``qubits`` in place."""
    m = np.ascontiguousarray(matrix, dtype=np.complex128)
    k = len(qubits)
    assert m.shape == (1 << k, 1 << k)
    lib().orc_apply_matrix_operator(_wf_ptr(wf), nqubits_of(wf),
                                    m.ctypes.data_as(_dp), k, _qubits(qubits))
    return wf


def apply_permutation(wf, perm, qubits):
    p = np.ascontiguousarray(perm, dtype=np.int64)
    lib().orc_apply_permutation(_wf_ptr(wf), nqubits_of(wf), len(qubits),
                                _qubits(qubits), p.ctypes.data_as(_i64p))
    return wf


def permutation_to_transpositions(perm):
    p = np.ascontiguousarray(perm, dtype=np.int64)
    a = (ctypes.c_int * len(p))()
    b = (ctypes.c_int * len(p))()
    n = lib().orc_permutation_to_transpositions(len(p), p.ctypes.data_as(_i64p), a, b)
    return [(a[i], b[i]) for i in range(n)]


def force_measurement(wf, measured_value, q, excited_probability):
    lib().orc_force_measurement(_wf_ptr(wf), nqubits_of(wf), measured_value, q,
                                excited_probability)
    return wf


def measure(wf, q, draw):
    """Returns (bit, draw_used, p1)."""
    used = ctypes.c_int(0)
    p1 = ctypes.c_double(0.0)
    bit = lib().orc_measure(_wf_ptr(wf), nqubits_of(wf), q, float(draw),
                            ctypes.byref(used), ctypes.byref(p1))
    return bit, bool(used.value), p1.value


def measure_compiled(wf, q, draw):
    p0 = ctypes.c_double(0.0)
    bit = lib().orc_measure_compiled(_wf_ptr(wf), nqubits_of(wf), q, float(draw),
                                     ctypes.byref(p0))
    return bit, p0.value


def sample_bisect(wf, p):
    return lib().orc_sample_bisect(_wf_ptr(wf), len(wf), float(p))


def measure_all(wf, draw):
    return lib().orc_measure_all(_wf_ptr(wf), nqubits_of(wf), float(draw))


def cdf(wf):
    out = np.zeros(len(wf), dtype=np.float64)
    lib().orc_cdf(_wf_ptr(wf), len(wf), out.ctypes.data_as(_dp))
    return out


def sample_multiple(wf, draws):
    d = np.ascontiguousarray(draws, dtype=np.float64)
    out = np.zeros(len(d), dtype=np.uint64)
    lib().orc_sample_multiple(_wf_ptr(wf), len(wf), d.ctypes.data_as(_dp), len(d),
                              out.ctypes.data_as(_u64p))
    return out


def inner(a, b):
    re = ctypes.c_double(0.0)
    im = ctypes.c_double(0.0)
    lib().orc_inner(_wf_ptr(a), _wf_ptr(b), len(a), ctypes.byref(re), ctypes.byref(im))
    return complex(re.value, im.value)


def gate_matrix(name: str, *params: float) -> np.ndarray:
    out = np.zeros(64, dtype=np.complex128)
    k = ctypes.c_int(0)
    pa = (ctypes.c_double * max(1, len(params)))(*params)
    rc = lib().orc_gate_matrix(name.encode(), pa, len(params),
                               out.ctypes.data_as(_dp), ctypes.byref(k))
    if rc != 0:
        raise KeyError(f"oracle has no gate {name} with {len(params)} parameters")
    d = 1 << k.value
    return out[: d * d].reshape(d, d).copy()


def run_gates(wf, gates):
    """Apply a list of (matrix, nat-tuple qubits) one gate at a time, the
    reference's per-gate apply-matrix-operator loop."""
    for m, qubits in gates:
        apply_matrix_operator(wf, m, qubits)
    return wf
