"""Continuous-batching request engine for the statevector path.

The reference's server (app/src/entry-point.lisp:655-673,
app/src/handle-request.lisp:44-187) runs one thread per HTTP connection,
each building its own QVM, with no batching across requests and a full GC
per request to release foreign memory.  Here requests are admitted onto the
GPU by HBM bytes (16*2^n for FP64, 8*2^n for FP32, plus scratch) within a
budget; every admitted request runs on its own state and CUDA stream, so the
device overlaps the work of many requests; a request that arrives while
others run is admitted as soon as a worker and enough memory are free.
Among the queued requests the cheapest one that fits goes first (estimated
cost = gates x 2^n, FP64 weighted by its slower arithmetic, divided by an
aging factor that grows with the wait), so small requests are not stuck
behind a 30-qubit FP64 job and large ones still progress.  A second lane of
workers takes only cheap requests, so that a small request does not wait for
a worker while every general worker holds a multi-second job; on the GPU
cheap requests run on high-priority streams while the others' tile passes
run as short CTAs, so the block scheduler interleaves them.  Freed states are
kept in a pool keyed by (qubits, precision) and
reused, evicted least-recently-used when admission needs their bytes.

Each request's result depends only on its own program and draws: states are
reset before use and every kernel is deterministic, so a request returns the
same shots alone and in the mix.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from .state import CudaPureState, Program, state_bytes

# States this small run as programs of a ProgramBatch: one persistent
# launch for every such request of a precision waiting at that moment.
SMALL_MAX_QUBITS = {"fp32": 13, "fp64": 12}


def is_small(req) -> bool:
    return req.n <= SMALL_MAX_QUBITS[req.precision] and all(len(q) <= 3 for _, q in req.gates)


@dataclass
class Request:
    n: int
    gates: list                   # (matrix, nat-tuple qubits) pairs
    shots: int
    precision: str = "fp32"
    draws: np.ndarray | None = None
    fused: bool = True
    tag: str = ""
    arrival: float = field(default_factory=time.perf_counter)


@dataclass
class Result:
    shots: np.ndarray
    queued_s: float
    run_s: float
    latency_s: float
    tag: str = ""


class StatePool:
    """Idle device states by (n, precision), least recently used first."""

    def __init__(self):
        self.idle = collections.OrderedDict()  # key -> list of states

    def take(self, n, prec):
        lst = self.idle.get((n, prec))
        if lst:
            s = lst.pop()
            if not lst:
                del self.idle[(n, prec)]
            return s
        return None

    def give(self, s: CudaPureState, prec):
        key = (s.num_qubits(), prec)
        self.idle.setdefault(key, []).append(s)
        self.idle.move_to_end(key)

    def evict_one(self, defer=None) -> int:
        """Remove the least recently used idle state and free it, or append it
        to `defer` for the caller to free outside its lock; returns its bytes
        (0 if none)."""
        if not self.idle:
            return 0
        key = next(iter(self.idle))
        lst = self.idle[key]
        s = lst.pop(0)
        if not lst:
            del self.idle[key]
        b = state_bytes(key[0], key[1])
        if defer is None:
            s.free()
        else:
            defer.append(s)
        return b

    def bytes(self) -> int:
        return sum(state_bytes(k[0], k[1]) * len(v) for k, v in self.idle.items())


class Server:
    def __init__(self, hbm_budget: float = 180e9, workers: int = 16, aging_s: float = 2.0,
                 fast_workers: int = 8, fast_cost: float = 1000.0 * (1 << 24),
                 reserve_pool: bool = True, small_batch: int = 64):
        """`workers` take any request; `fast_workers` more take only requests
        whose estimated cost (gates x 2^n, FP64 x 8) is at most `fast_cost`
        (by default a 1000-gate 24-qubit FP32 program), so that a small
        request never waits for a worker held by a multi-second job.
        `reserve_pool` maps the budget into the device memory pool at start.
        A worker that admits a small request (<= 13 qubits in FP32, <= 12 in
        FP64, gates of <= 3 qubits) takes up to `small_batch` - 1 more small
        requests of that precision from the queue and runs them all as one
        ProgramBatch launch (0: every request runs on its own state)."""
        self.small_batch = int(small_batch)
        self.budget = int(hbm_budget)
        self.aging_s = float(aging_s)
        self.fast_cost = float(fast_cost)
        if reserve_pool and workers + fast_workers > 0:
            # map the budget's device memory once: growing the pool while
            # requests run stalls the workers' CUDA calls
            from . import _lib as L
            L.lib().qvmg_device_reserve(int(self.budget))  # best effort
        self.reserved = 0              # bytes of running requests + idle pooled states
        self.pool = StatePool()
        self.queue = collections.deque()
        self.cv = threading.Condition()
        self.stop = False
        self.threads = [threading.Thread(target=self._worker, args=(False,), daemon=True)
                        for _ in range(workers)]
        self.threads += [threading.Thread(target=self._worker, args=(True,), daemon=True)
                         for _ in range(fast_workers)]
        for t in self.threads:
            t.start()

    def submit(self, req: Request) -> Future:
        need = state_bytes(req.n, req.precision)
        if need == 0 or need > self.budget:
            raise ValueError(f"a {req.n}-qubit {req.precision} state does not fit the "
                             f"{self.budget} byte budget")
        fut = Future()
        with self.cv:
            self.queue.append((req, fut, need))
            # every waiting worker: one of the fast lane may not take this request
            self.cv.notify_all()
        return fut

    @staticmethod
    def cost(req: Request) -> float:
        """Estimated device work: gates x amplitudes, FP64 weighted by its
        slower arithmetic on this part."""
        return len(req.gates) * float(1 << req.n) * (8.0 if req.precision == "fp64" else 1.0)

    def _order(self):
        """Queue positions, cheapest first with aging: a request's cost is
        divided by (1 + wait / aging_s), so large jobs are not starved."""
        now = time.perf_counter()
        score = [self.cost(r) / (1.0 + max(0.0, now - r.arrival) / self.aging_s)
                 for r, _, _ in self.queue]
        return sorted(range(len(self.queue)), key=score.__getitem__)

    def _admit(self, fast_only: bool = False, evicted=None):
        """The cheapest (aged) queued request that fits, evicting idle pooled
        states if that makes it fit (into `evicted`, freed by the caller after
        it drops the lock); a fast worker takes only cheap requests.  Called
        with the lock held."""
        for i in self._order():
            req, fut, need = self.queue[i]
            if fast_only and self.cost(req) > self.fast_cost:
                continue
            key_state = self.pool.take(req.n, req.precision)
            if key_state is not None:
                del self.queue[i]
                return req, fut, need, key_state   # its bytes are already reserved
            while self.reserved + need > self.budget:
                freed = self.pool.evict_one(evicted)
                if freed == 0:
                    break
                self.reserved -= freed
            if self.reserved + need <= self.budget:
                del self.queue[i]
                self.reserved += need
                return req, fut, need, None
        return None

    def _worker(self, fast_only: bool = False):
        while True:
            evicted = []
            with self.cv:
                item = None
                while not self.stop:
                    item = self._admit(fast_only, evicted)
                    if item is not None or evicted:
                        break
                    self.cv.wait()
            # Evicted states are freed outside the lock.  Their bytes were
            # released from the budget already: this request's state is
            # created below, after these frees.
            for s in evicted:
                s.free()
            if item is None:
                if evicted and not self.stop:
                    with self.cv:  # budget was freed: other lanes may admit now
                        self.cv.notify_all()
                    continue
                return
            req, fut, need, st = item
            if self.small_batch > 0 and is_small(req):
                self._run_small_batch(req, fut, need, st)
                continue
            t0 = time.perf_counter()
            try:
                if st is None:
                    st = CudaPureState(req.n, req.precision)
                else:
                    st.set_to_zero_state()
                # cheap requests on a high-priority stream; the others yield
                # (their tile passes run as short CTAs)
                st.set_priority(1 if self.cost(req) <= self.fast_cost else -1)
                prog = Program()
                try:  # the plan's device buffers are freed on every path
                    prog.add_gates(req.gates)
                    if req.fused:
                        prog.plan(req.n, req.precision, fused=True, fusion_width=2)
                    prog.run(st, fused=req.fused)
                    draws = req.draws
                    if draws is None:
                        draws = np.random.default_rng(0).random(req.shots)
                    shots = st.sample(draws)
                finally:
                    prog.free()
                t1 = time.perf_counter()
                fut.set_result(Result(shots, t0 - req.arrival, t1 - t0, t1 - req.arrival, req.tag))
            except Exception as e:  # the request fails, the server keeps going
                fut.set_exception(e)
                if st is not None:
                    st.free()
                    st = None
            with self.cv:
                if st is not None:
                    self.pool.give(st, req.precision)   # stays reserved while pooled
                else:
                    self.reserved -= need
                self.cv.notify_all()

    def _run_small_batch(self, req, fut, need, st):
        """Run `req` with the small requests of its precision that are still
        queued (up to small_batch in all) as one ProgramBatch launch."""
        from .batch import ProgramBatch
        group = [(req, fut, need)]
        with self.cv:
            keep = collections.deque()
            while self.queue:
                item = self.queue.popleft()
                r = item[0]
                if (len(group) < self.small_batch and r.precision == req.precision
                        and is_small(r) and self.reserved + item[2] <= self.budget):
                    group.append(item)
                    self.reserved += item[2]
                else:
                    keep.append(item)
            self.queue = keep
        t0 = time.perf_counter()
        try:
            draws = [r.draws if r.draws is not None else np.random.default_rng(0).random(r.shots)
                     for r, _, _ in group]
            b = ProgramBatch([(r.n, r.gates, r.shots) for r, _, _ in group], req.precision)
            try:
                shots = b.run(draws)
            finally:
                b.free()
            t1 = time.perf_counter()
            for (r, f, _), sh in zip(group, shots):
                f.set_result(Result(sh, t0 - r.arrival, t1 - t0, t1 - r.arrival, r.tag))
        except Exception as e:  # the batch's requests fail, the server keeps going
            for _, f, _ in group:
                if not f.done():
                    f.set_exception(e)
        with self.cv:
            if st is not None:
                self.pool.give(st, req.precision)   # the admitted state stays pooled
            else:
                self.reserved -= need
            for _, _, nd in group[1:]:
                self.reserved -= nd
            self.cv.notify_all()

    def close_now(self):
        """Cancel the queued requests, let running ones finish, free states."""
        with self.cv:
            while self.queue:
                _, fut, _ = self.queue.popleft()
                fut.cancel()
        self.close()

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        with self.cv:
            while self.pool.evict_one():
                pass
            self.reserved = 0


def serving_workload(duration_s: float, rate: float = 200.0, seed: int = 5,
                     nmin: int = 10, nmax: int = 30, depth=(5, 40)):
    """The serving stream: Poisson arrivals, qubit counts uniform in
    [nmin, nmax], programs drawn from the random-layer family, the QFT and
    QAOA MaxCut (depth uniform in `depth`), shots log-uniform in 1..10^4,
    FP32 or FP64 per request.  Returns [(arrival_offset_s, Request)]."""
    from . import circuits
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration_s:
            return out
        n = int(rng.integers(nmin, nmax + 1))
        fam = ["layers", "qft", "qaoa"][int(rng.integers(3))]
        d = int(rng.integers(depth[0], depth[1] + 1))
        if fam == "layers":
            gates = circuits.random_layers(n, layers=d, seed=int(rng.integers(1 << 30)))
        elif fam == "qft":
            gates = circuits.qft(n)
        else:
            m = n if n % 2 == 0 else n - 1
            edges = circuits.random_3_regular_graph(m, rng)
            p = max(1, d // 10)
            gates = circuits.qaoa_maxcut(m, edges, rng.uniform(0, np.pi, p),
                                         rng.uniform(0, np.pi / 2, p))
        shots = int(np.exp(rng.uniform(0, np.log(1e4))))
        prec = "fp32" if rng.random() < 0.5 else "fp64"
        draws = rng.random(shots)
        out.append((t, Request(n, gates, shots, prec, draws, True, f"{fam}-{n}-{prec}")))
