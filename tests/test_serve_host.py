"""Host logic of the serving engine's admission (no GPU): cheapest request
first with aging, the fast lane taking only cheap requests, and the HBM
budget.  No worker threads are started."""
import time
from concurrent.futures import Future

import numpy as np
import pytest

from qvm_gb300 import circuits
from qvm_gb300.serve import Request, Server
from qvm_gb300.state import state_bytes


def _server(budget=100e9):
    return Server(hbm_budget=budget, workers=0, fast_workers=0,
                  fast_cost=1000.0 * (1 << 24))


def _queue(srv, reqs):
    for r in reqs:
        srv.queue.append((r, Future(), state_bytes(r.n, r.precision)))


def test_cheapest_first_and_fast_lane():
    srv = _server()
    big = Request(28, circuits.qft(28), 10, "fp64")
    small = Request(12, circuits.qft(12), 10, "fp32")
    _queue(srv, [big, small])
    # a fast worker skips the 28-qubit FP64 job
    req, _, need, st = srv._admit(fast_only=True)
    assert req is small and st is None and srv.reserved == need
    # nothing cheap is left for the fast lane; a general worker takes the big one
    assert srv._admit(fast_only=True) is None
    req, _, _, _ = srv._admit(fast_only=False)
    assert req is big
    assert not srv.queue


def test_aging_lets_a_large_job_overtake():
    srv = _server()
    big = Request(24, circuits.qft(24), 1, "fp32")
    small = Request(20, circuits.qft(20), 1, "fp32")
    big.arrival = time.perf_counter() - 60.0   # waited a minute
    _queue(srv, [small, big])
    assert srv._admit()[0] is big


def test_budget_holds_back_what_does_not_fit():
    need = state_bytes(20, "fp64")
    srv = _server(budget=need * 1.5)
    _queue(srv, [Request(20, circuits.qft(20), 1, "fp64"), Request(20, circuits.qft(20), 1, "fp64")])
    assert srv._admit() is not None
    assert srv._admit() is None          # the second does not fit beside the first
    assert srv.reserved <= srv.budget


class _FakeState:
    """Stands in for a device state: tracks live bytes, records priorities."""
    lock = None
    live = 0
    peak = 0

    def __init__(self, n, prec):
        self.n, self.prec, self.prio = n, prec, 0
        with _FakeState.lock:
            _FakeState.live += state_bytes(n, prec)
            _FakeState.peak = max(_FakeState.peak, _FakeState.live)

    def num_qubits(self):
        return self.n

    def set_to_zero_state(self):
        pass

    def set_priority(self, p):
        self.prio = p

    def sample(self, draws):
        time.sleep(0.002)
        return np.floor(np.asarray(draws) * (1 << self.n)).astype(np.int64) * 2 + (self.prio > 0)

    def free(self):
        with _FakeState.lock:
            _FakeState.live -= state_bytes(self.n, self.prec)


class _FakeProgram:
    def add_gates(self, gates):
        self.ng = len(gates)
        return self

    def plan(self, *a, **k):
        pass

    def run(self, st, fused=True):
        time.sleep(0.001 * (1 + st.n % 3))

    def free(self):
        pass


def test_workers_lanes_eviction_and_priority(monkeypatch):
    """The worker loop with fake states: every request completes with its
    own result, cheap ones on the fast lane's high priority and the others
    yielding, pooled states are evicted within the budget."""
    import threading
    from qvm_gb300 import serve
    monkeypatch.setattr(serve, "CudaPureState", _FakeState)
    monkeypatch.setattr(serve, "Program", _FakeProgram)
    _FakeState.lock = threading.Lock()
    _FakeState.live = _FakeState.peak = 0
    budget = 3 * state_bytes(20, "fp64")
    fast_cost = 200.0 * (1 << 14)
    srv = Server(hbm_budget=budget, workers=3, fast_workers=2, fast_cost=fast_cost,
                 reserve_pool=False, small_batch=0)
    rng = np.random.default_rng(8)
    reqs = []
    for i in range(60):
        n = int(rng.choice([10, 12, 14, 18, 20]))
        prec = "fp32" if i % 2 else "fp64"
        gates = [None] * int(rng.integers(5, 300))
        reqs.append(Request(n, gates, 16, prec, rng.random(16), True, f"r{i}"))
    futs = [(r, srv.submit(r)) for r in reqs]
    for r, f in futs:
        res = f.result(timeout=60)
        high = Server.cost(r) <= fast_cost
        want = np.floor(r.draws * (1 << r.n)).astype(np.int64) * 2 + int(high)
        np.testing.assert_array_equal(res.shots, want)
    assert srv.reserved <= budget
    srv.close()
    assert _FakeState.live == 0                      # everything freed at close
    # evicted states are freed outside the lock, so new states may briefly
    # overlap them: at most one evicted state per worker (5) beyond the budget
    assert _FakeState.peak <= budget + 5 * state_bytes(20, "fp64")


def test_failed_request_frees_its_program(monkeypatch):
    """A request whose run raises fails alone: its Program's device plan is
    still freed, its state is released from the budget, and the server keeps
    serving the next request."""
    import threading
    from qvm_gb300 import serve

    class _Counting(_FakeProgram):
        made = 0
        freed = 0

        def __init__(self):
            _Counting.made += 1

        def run(self, st, fused=True):
            if self.ng == 13:
                raise RuntimeError("planted run failure")

        def free(self):
            _Counting.freed += 1

    monkeypatch.setattr(serve, "CudaPureState", _FakeState)
    monkeypatch.setattr(serve, "Program", _Counting)
    _FakeState.lock = threading.Lock()
    _FakeState.live = _FakeState.peak = 0
    srv = Server(hbm_budget=4 * state_bytes(14, "fp64"), workers=2, fast_workers=0,
                 reserve_pool=False, small_batch=0)
    bad = srv.submit(Request(12, [None] * 13, 4, "fp64", np.zeros(4), True, "bad"))
    good = srv.submit(Request(12, [None] * 5, 4, "fp64", np.zeros(4), True, "good"))
    with pytest.raises(RuntimeError, match="planted"):
        bad.result(timeout=30)
    assert good.result(timeout=30).tag == "good"
    srv.close()
    assert _Counting.made == 2 and _Counting.freed == 2
    assert _FakeState.live == 0


def test_small_requests_run_as_batches(monkeypatch):
    """Small requests waiting together run as one ProgramBatch per precision
    (a fake here): every request gets its own program's shots, large ones
    keep their own states, and the budget returns to zero."""
    import threading
    from qvm_gb300 import batch, serve

    calls = []

    class _FakeBatch:
        def __init__(self, programs, precision):
            self.programs, self.precision = programs, precision
            calls.append((len(programs), precision))

        def run(self, draws):
            time.sleep(0.01)
            return [np.full(k, n * 1000 + len(g), dtype=np.uint64)
                    for (n, g, k) in self.programs]

        def free(self):
            pass

    monkeypatch.setattr(batch, "ProgramBatch", _FakeBatch)
    monkeypatch.setattr(serve, "CudaPureState", _FakeState)
    monkeypatch.setattr(serve, "Program", _FakeProgram)
    _FakeState.lock = threading.Lock()
    _FakeState.live = _FakeState.peak = 0
    srv = Server(hbm_budget=4 * state_bytes(20, "fp64"), workers=1, fast_workers=0,
                 reserve_pool=False, small_batch=8)
    g1 = [(np.eye(2), [0])]
    reqs = [Request(20, [None] * 3, 2, "fp32", np.zeros(2), True, "big")]
    reqs += [Request(10 + i % 3, g1 * (i + 1), 3, "fp32" if i % 2 else "fp64", np.zeros(3),
                     True, f"s{i}") for i in range(12)]
    futs = [(r, srv.submit(r)) for r in reqs]
    for r, f in futs:
        res = f.result(timeout=30)
        if r.tag != "big":
            assert (res.shots == r.n * 1000 + len(r.gates)).all(), r.tag
    srv.close()
    assert sum(c for c, _ in calls) == 12 and len(calls) < 12   # batched, both precisions
    assert {p for _, p in calls} == {"fp32", "fp64"}
    assert srv.reserved == 0
