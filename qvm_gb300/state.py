"""Device-resident pure state and gate programs over the C ABI.

``CudaPureState`` mirrors the reference's state protocol on ``pure-state``
(src/state-representation.lisp:25-168): ``num_qubits``,
``set_to_zero_state``, ``state_elements`` / ``set_state_elements`` (the
amplitudes, downloaded/uploaded as complex128, LSB-first), plus the
measurement protocol of src/measurement.lisp.  The amplitudes never leave
HBM unless ``state_elements`` is called.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L

PRECISIONS = {"fp64": L.FP64, "fp32": L.FP32, L.FP64: L.FP64, L.FP32: L.FP32}


def _qubit_array(qubits):
    return (ctypes.c_int * len(qubits))(*[int(q) for q in qubits])


def _cplx(arr) -> np.ndarray:
    return np.ascontiguousarray(arr, dtype=np.complex128)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def state_bytes(nqubits: int, precision="fp64") -> int:
    """HBM bytes a state of this size needs (admission control)."""
    return int(L.lib().qvmg_state_bytes(int(nqubits), PRECISIONS[precision]))


def device_info():
    sms = ctypes.c_int(0)
    free = ctypes.c_uint64(0)
    total = ctypes.c_uint64(0)
    L.call("qvmg_device_info", ctypes.byref(sms), ctypes.byref(free), ctypes.byref(total))
    return {"sm_count": sms.value, "free_bytes": free.value, "total_bytes": total.value}


class CudaPureState:
    """A pure state of ``num_qubits`` qubits held in GPU memory."""

    def __init__(self, num_qubits: int, precision="fp64"):
        self._h = ctypes.c_void_p()
        self.precision = PRECISIONS[precision]
        L.call("qvmg_state_create", int(num_qubits), self.precision, ctypes.byref(self._h))
        self._n = int(num_qubits)

    # -- lifecycle ----------------------------------------------------------
    @property
    def handle(self):
        if not self._h:
            raise ValueError("state has been freed")
        return self._h

    def free(self):
        if self._h:
            L.call("qvmg_state_free", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    # -- state protocol ------------------------------------------------------
    def num_qubits(self) -> int:
        return self._n

    def set_to_zero_state(self):
        L.call("qvmg_state_reset", self.handle)

    def state_elements(self) -> np.ndarray:
        out = np.empty(1 << self._n, dtype=np.complex128)
        L.call("qvmg_state_download", self.handle, _dptr(out))
        return out

    def set_state_elements(self, amps):
        a = _cplx(amps)
        if a.shape != (1 << self._n,):
            raise ValueError(f"expected {1 << self._n} amplitudes, got {a.shape}")
        L.call("qvmg_state_upload", self.handle, _dptr(a))

    def copy_from(self, other: "CudaPureState"):
        L.call("qvmg_state_copy", self.handle, other.handle)

    def set_priority(self, priority: int):
        """Scheduling class on a shared GPU: 1 high-priority stream, 0
        default, -1 yield (tile passes in short CTAs).  Results do not
        depend on it."""
        L.call("qvmg_state_set_priority", self.handle, int(priority))

    def sync(self):
        L.call("qvmg_state_sync", self.handle)

    def stream(self) -> int:
        """The state's cudaStream_t as an integer (for events / ordering)."""
        p = ctypes.c_void_p()
        L.call("qvmg_state_stream", self.handle, ctypes.byref(p))
        return int(p.value or 0)

    # -- gates -----------------------------------------------------------------
    def apply_matrix(self, matrix, qubits):
        """apply-matrix-operator: ``qubits`` is a nat-tuple (qubits[0] is
        the matrix LSB, i.e. the last Quil argument)."""
        m = _cplx(matrix)
        L.call("qvmg_apply_dense", self.handle, len(qubits), _qubit_array(qubits), _dptr(m))

    def apply_permutation(self, perm, qubits):
        p = np.ascontiguousarray(perm, dtype=np.int64)
        L.call("qvmg_apply_permutation", self.handle, len(qubits), _qubit_array(qubits),
               p.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))

    def apply_diagonal(self, diag, qubits):
        d = _cplx(diag)
        L.call("qvmg_apply_diagonal", self.handle, len(qubits), _qubit_array(qubits), _dptr(d))

    # -- noise ---------------------------------------------------------------------
    def reduced_density_matrix(self, qubits) -> np.ndarray:
        """rho of 1 or 2 qubits (nat order: bit j of an index <-> qubits[j])."""
        d = 1 << len(qubits)
        out = np.empty((d, d), dtype=np.complex128)
        L.call("qvmg_reduced_density_matrix", self.handle, len(qubits), _qubit_array(qubits),
               _dptr(out))
        return out

    def density_diagonal(self) -> np.ndarray:
        """Re rho[i][i] of a density matrix held as vec(rho) (2n qubits)."""
        out = np.empty(1 << (self._n // 2), dtype=np.float64)
        L.call("qvmg_density_diagonal", self.handle, _dptr(out))
        return out

    def apply_kraus(self, kraus_ops, qubits, draw: float):
        """Stochastic Kraus map on 1 or 2 qubits; returns (chosen index, p_j)."""
        ops = np.ascontiguousarray(np.stack([_cplx(k) for k in kraus_ops]))
        chosen = ctypes.c_int(-1)
        prob = ctypes.c_double(0.0)
        L.call("qvmg_apply_kraus", self.handle, len(qubits), _qubit_array(qubits), len(ops),
               _dptr(ops), float(draw), ctypes.byref(chosen), ctypes.byref(prob))
        return chosen.value, prob.value

    # -- measurement -------------------------------------------------------------
    def excited_probability(self, q: int) -> float:
        p = ctypes.c_double()
        L.call("qvmg_prob_excited", self.handle, int(q), ctypes.byref(p))
        return p.value

    def ground_probability(self, q: int) -> float:
        p = ctypes.c_double()
        L.call("qvmg_prob_ground", self.handle, int(q), ctypes.byref(p))
        return p.value

    def force_measurement(self, measured_value: int, q: int, excited_probability: float):
        L.call("qvmg_force_measurement", self.handle, int(q), int(measured_value),
               float(excited_probability))

    def measure(self, q: int, draw: float, compiled: bool = False):
        """Returns (bit, draw_used, probability)."""
        bit = ctypes.c_int()
        used = ctypes.c_int()
        prob = ctypes.c_double()
        conv = L.MEASURE_COMPILED if compiled else L.MEASURE_INTERPRETED
        L.call("qvmg_measure", self.handle, int(q), float(draw), conv, ctypes.byref(bit),
               ctypes.byref(used), ctypes.byref(prob))
        return bit.value, bool(used.value), prob.value

    def measure_all(self, draw: float) -> int:
        idx = ctypes.c_uint64()
        L.call("qvmg_measure_all", self.handle, float(draw), ctypes.byref(idx))
        return int(idx.value)

    def sample(self, draws, rule: str = "bisect") -> np.ndarray:
        d = np.ascontiguousarray(draws, dtype=np.float64)
        out = np.zeros(len(d), dtype=np.uint64)
        r = L.SAMPLE_BISECT if rule == "bisect" else L.SAMPLE_CDF
        L.call("qvmg_sample", self.handle, _dptr(d), len(d), r,
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return out

    def probabilities(self) -> np.ndarray:
        out = np.empty(1 << self._n, dtype=np.float64)
        L.call("qvmg_probabilities", self.handle, _dptr(out))
        return out

    def marginal_probabilities(self, qubits) -> np.ndarray:
        """out[m] = P(bit qubits[j] = bit j of m for every j); <= 20 qubits."""
        out = np.empty(1 << len(qubits), dtype=np.float64)
        L.call("qvmg_marginal_probabilities", self.handle, len(qubits), _qubit_array(qubits),
               _dptr(out))
        return out

    def measure_sequence(self, qubits, draws, ntrials: int, compiled: bool = False):
        """Measure ``qubits`` in order (-1 = unused slot) on ``ntrials``
        reloads of this state; returns (bits[ntrials, len(qubits)], draws
        consumed).  The state is not modified."""
        d = np.ascontiguousarray(draws, dtype=np.float64)
        bits = np.zeros((int(ntrials), len(qubits)), dtype=np.uint8)
        used = ctypes.c_uint64(0)
        conv = L.MEASURE_COMPILED if compiled else L.MEASURE_INTERPRETED
        L.call("qvmg_measure_sequence", self.handle, len(qubits), _qubit_array(qubits), conv,
               int(ntrials), _dptr(d), len(d), bits.ctypes.data_as(ctypes.c_void_p),
               ctypes.byref(used))
        return bits, int(used.value)

    def wavefunction_octets(self) -> memoryview:
        """The amplitudes as big-endian complex doubles (16 octets each), as a
        bytes-like view of the host buffer they were written into."""
        out = np.empty(16 << self._n, dtype=np.uint8)
        L.call("qvmg_wavefunction_octets", self.handle, out.ctypes.data_as(ctypes.c_void_p))
        return memoryview(out)

    def probabilities_octets(self) -> memoryview:
        """|a_i|^2 as big-endian doubles (8 octets each), bytes-like."""
        out = np.empty(8 << self._n, dtype=np.uint8)
        L.call("qvmg_probabilities_octets", self.handle, out.ctypes.data_as(ctypes.c_void_p))
        return memoryview(out)

    def norm(self) -> float:
        n = ctypes.c_double()
        L.call("qvmg_norm", self.handle, ctypes.byref(n))
        return n.value

    def normalize(self):
        L.call("qvmg_normalize", self.handle)

    def inner(self, other: "CudaPureState") -> complex:
        re = ctypes.c_double()
        im = ctypes.c_double()
        L.call("qvmg_inner", self.handle, other.handle, ctypes.byref(re), ctypes.byref(im))
        return complex(re.value, im.value)

    def fidelity(self, other: "CudaPureState"):
        """(|<self|other>|^2, max |self_i - other_i|)."""
        f = ctypes.c_double()
        e = ctypes.c_double()
        L.call("qvmg_fidelity", self.handle, other.handle, ctypes.byref(f), ctypes.byref(e))
        return f.value, e.value


class Program:
    """A list of gate ops run on a state in plain or fused mode."""

    def __init__(self):
        self._h = ctypes.c_void_p()
        # bumped by every added op: tuned choices cached for an older op list
        # are not reused
        self.generation = 0
        L.call("qvmg_program_create", ctypes.byref(self._h))

    def free(self):
        if self._h:
            L.call("qvmg_program_free", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def add_dense(self, matrix, qubits):
        m = _cplx(matrix)
        self.generation += 1
        L.call("qvmg_program_add_dense", self._h, len(qubits), _qubit_array(qubits), _dptr(m))

    def add_permutation(self, perm, qubits):
        p = np.ascontiguousarray(perm, dtype=np.int64)
        self.generation += 1
        L.call("qvmg_program_add_permutation", self._h, len(qubits), _qubit_array(qubits),
               p.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))

    def add_diagonal(self, diag, qubits):
        d = _cplx(diag)
        self.generation += 1
        L.call("qvmg_program_add_diagonal", self._h, len(qubits), _qubit_array(qubits), _dptr(d))

    def add_gates(self, gates):
        """Add (matrix, nat-tuple qubits) pairs as dense ops, in one call."""
        gates = list(gates)
        if not gates:
            return self
        ks = np.fromiter((len(qs) for _, qs in gates), dtype=np.int32, count=len(gates))
        qubits = np.fromiter((int(q) for _, qs in gates for q in qs), dtype=np.int32,
                             count=int(ks.sum()))
        mats = np.concatenate([np.asarray(m, dtype=np.complex128).ravel() for m, _ in gates])
        ip = ctypes.POINTER(ctypes.c_int)
        self.generation += 1
        L.call("qvmg_program_add_dense_many", self._h, len(gates), ks.ctypes.data_as(ip),
               qubits.ctypes.data_as(ip), _dptr(mats))
        return self

    def set_register_stages(self, enable: bool):
        """Apply runs of 1-/2-qubit blocks in registers inside FP32 tiles."""
        L.call("qvmg_program_set_option", self._h, 1, 1 if enable else 0)

    def set_tensor_cores(self, enable: bool):
        """Merge the dense blocks of FP32 tiles into blocks of up to
        min(5, max(3, fusion_width)) qubits and run the 3- to 5-qubit ones as
        tcgen05 MMAs in bf16x3 split precision (three bf16 products per
        FP32 product, FP32 accumulation)."""
        L.call("qvmg_program_set_option", self._h, 2, 1 if enable else 0)

    def num_ops(self) -> int:
        n = ctypes.c_int()
        L.call("qvmg_program_num_ops", self._h, ctypes.byref(n))
        return n.value

    def plan(self, nqubits: int, precision="fp64", fused: bool = True, fusion_width: int = 2,
             tile_qubits: int = 0) -> dict:
        """Plan on the host (no GPU work) and return the plan statistics."""
        npasses = ctypes.c_int()
        L.call("qvmg_program_plan", self._h, int(nqubits), PRECISIONS[precision],
               L.RUN_FUSED if fused else L.RUN_PLAIN, int(fusion_width), int(tile_qubits),
               ctypes.byref(npasses))
        st = (ctypes.c_int64 * 8)()
        L.call("qvmg_program_plan_stats", self._h, st, 8)
        keys = ["source_ops", "passes", "tile_passes", "fused_blocks", "diag_passes",
                "perm_passes", "bytes_moved", "upload_bytes"]
        return dict(zip(keys, [int(x) for x in st]))

    def describe(self) -> dict:
        """The last plan's passes as a dict (see qvmg_program_plan_describe)."""
        import json
        need = ctypes.c_uint64()
        L.call("qvmg_program_plan_describe", self._h, None, 0, ctypes.byref(need))
        buf = ctypes.create_string_buffer(need.value)
        L.call("qvmg_program_plan_describe", self._h, buf, need.value, ctypes.byref(need))
        return json.loads(buf.value.decode())

    def run(self, state: CudaPureState, fused: bool = True):
        L.call("qvmg_program_run", state.handle, self._h, L.RUN_FUSED if fused else L.RUN_PLAIN)

    def run_profiled(self, state: CudaPureState, fused: bool = True, cap: int = 1 << 16):
        """Run with an event around every pass; returns (ms[], kinds[]) with
        kinds 0 dense, 1 diagonal, 2 permutation, 3 tile."""
        ms = (ctypes.c_float * cap)()
        kinds = (ctypes.c_int * cap)()
        n = ctypes.c_int()
        L.call("qvmg_program_run_profiled", state.handle, self._h,
               L.RUN_FUSED if fused else L.RUN_PLAIN, ms, kinds, cap, ctypes.byref(n))
        k = min(n.value, cap)
        return np.array(ms[:k], dtype=np.float64), np.array(kinds[:k], dtype=np.int32)
