"""Batched circuits in one persistent launch: QAOA MaxCut instances, and
batches of arbitrary small programs.

Mirrors the QAOA workload of the reference's examples/qaoa.lisp:7-206 (H on
all qubits, p layers of ZZ(gamma) on graph edges and RX(2 beta) on all
qubits; sampling with sample-wavefunction-multiple-times), for batches of
uneven instances held on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L


class QaoaBatch:
    def __init__(self, graphs, gammas, betas):
        """graphs: list of (n, edges); gammas, betas: (ninst, p) arrays."""
        self.ninst = len(graphs)
        g = np.ascontiguousarray(gammas, dtype=np.float64).reshape(self.ninst, -1)
        b = np.ascontiguousarray(betas, dtype=np.float64).reshape(self.ninst, -1)
        if g.shape != b.shape:
            raise ValueError("gammas and betas must have the same shape")
        self.p = g.shape[1]
        self.n = np.array([int(n) for n, _ in graphs], dtype=np.int32)
        ne = np.array([len(e) for _, e in graphs], dtype=np.int32)
        flat = np.array([x for _, e in graphs for uv in e for x in uv], dtype=np.int32)
        if flat.size == 0:
            flat = np.zeros(2, dtype=np.int32)
        self.graphs = [(int(n), [tuple(map(int, uv)) for uv in e]) for n, e in graphs]
        self._h = ctypes.c_void_p()
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.call("qvmg_qaoa_batch_create", self.ninst, self.n.ctypes.data_as(ip),
               ne.ctypes.data_as(ip), flat.ctypes.data_as(ip), self.p, g.ctypes.data_as(dp),
               b.ctypes.data_as(dp), ctypes.byref(self._h))

    def set_angles(self, gammas, betas):
        g = np.ascontiguousarray(gammas, dtype=np.float64).reshape(self.ninst, self.p)
        b = np.ascontiguousarray(betas, dtype=np.float64).reshape(self.ninst, self.p)
        dp = ctypes.POINTER(ctypes.c_double)
        L.call("qvmg_qaoa_batch_set_angles", self._h, g.ctypes.data_as(dp), b.ctypes.data_as(dp))

    def run(self, draws=None):
        """Returns (expectations[ninst], shots[ninst, nshots] or None)."""
        dp = ctypes.POINTER(ctypes.c_double)
        ex = np.zeros(self.ninst, dtype=np.float64)
        if draws is None:
            L.call("qvmg_qaoa_batch_run", self._h, None, 0, ex.ctypes.data_as(dp), None)
            return ex, None
        d = np.ascontiguousarray(draws, dtype=np.float64).reshape(self.ninst, -1)
        shots = np.zeros(d.shape, dtype=np.uint32)
        L.call("qvmg_qaoa_batch_run", self._h, d.ctypes.data_as(dp), d.shape[1],
               ex.ctypes.data_as(dp), shots.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        return ex, shots

    def state(self, i: int) -> np.ndarray:
        out = np.zeros(1 << int(self.n[i]), dtype=np.complex128)
        L.call("qvmg_qaoa_batch_state", self._h, int(i),
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def device_bytes(self) -> int:
        return int(L.lib().qvmg_qaoa_batch_bytes(self._h))

    def free(self):
        if self._h:
            L.call("qvmg_qaoa_batch_free", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ProgramBatch:
    """Many small programs (gate lists on 1..13 qubits in FP32, 1..12 in
    FP64) run from |0...0> in one persistent launch, each with its own
    shots.  programs: list of (n, gates, nshots), gates a list of
    (matrix, nat-tuple qubits) with 1- to 3-qubit matrices."""

    def __init__(self, programs, precision: str = "fp64"):
        from .state import PRECISIONS
        self.nprog = len(programs)
        self.n = np.array([int(n) for n, _, _ in programs], dtype=np.int32)
        self.nshots = np.array([int(k) for _, _, k in programs], dtype=np.int32)
        nops = np.array([len(g) for _, g, _ in programs], dtype=np.int32)
        ks, qs, ms = [], [], []
        for _, gates, _ in programs:
            for m, q in gates:
                ks.append(len(q))
                qs.extend(int(x) for x in q)
                ms.append(np.asarray(m, dtype=np.complex128).ravel())
        op_k = np.array(ks or [0], dtype=np.int32)
        op_q = np.array(qs or [0], dtype=np.int32)
        mats = np.concatenate(ms) if ms else np.zeros(1, dtype=np.complex128)
        mats = np.ascontiguousarray(mats.view(np.float64))
        ip = ctypes.POINTER(ctypes.c_int)
        self._h = ctypes.c_void_p()
        L.call("qvmg_sbatch_create", PRECISIONS[precision], self.nprog,
               self.n.ctypes.data_as(ip), nops.ctypes.data_as(ip), op_k.ctypes.data_as(ip),
               op_q.ctypes.data_as(ip), mats.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
               self.nshots.ctypes.data_as(ip), ctypes.byref(self._h))
        self.offsets = []
        off = ctypes.c_uint64()
        for i in range(self.nprog):
            L.call("qvmg_sbatch_shot_offset", self._h, i, ctypes.byref(off))
            self.offsets.append(int(off.value))

    def run(self, draws):
        """draws: one array per program (its nshots uniforms).  Returns the
        list of per-program shot index arrays."""
        flat = np.concatenate([np.asarray(d, dtype=np.float64).ravel() for d in draws]) \
            if self.nprog else np.zeros(0)
        if len(flat) != int(self.nshots.sum()):
            raise ValueError("one draw per shot of every program is required")
        flat = np.ascontiguousarray(flat)
        out = np.zeros(max(1, len(flat)), dtype=np.uint64)
        L.call("qvmg_sbatch_run", self._h, flat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return [out[o:o + int(k)].copy() for o, k in zip(self.offsets, self.nshots)]

    def state(self, i: int) -> np.ndarray:
        out = np.zeros(1 << int(self.n[i]), dtype=np.complex128)
        L.call("qvmg_sbatch_state", self._h, int(i),
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def free(self):
        if self._h:
            L.call("qvmg_sbatch_free", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def random_qaoa_batch(ngraphs: int, sizes, params_per_graph: int, p: int, seed: int = 4):
    """The batched QAOA workload: random 3-regular graphs with n drawn from
    `sizes`, each with `params_per_graph` (gamma, beta) sets drawn uniformly
    from [0, pi) x [0, pi/2); returns (graphs, gammas, betas)."""
    from .circuits import random_3_regular_graph
    rng = np.random.default_rng(seed)
    graphs, gam, bet = [], [], []
    for _ in range(ngraphs):
        n = int(rng.choice(sizes))
        edges = random_3_regular_graph(n, rng)
        for _ in range(params_per_graph):
            graphs.append((n, edges))
            gam.append(rng.uniform(0, np.pi, p))
            bet.append(rng.uniform(0, np.pi / 2, p))
    return graphs, np.array(gam), np.array(bet)
