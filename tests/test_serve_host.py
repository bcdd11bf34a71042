"""Host logic of the serving engine's admission (no GPU): cheapest request
first with aging, the fast lane taking only cheap requests, and the HBM
budget.  No worker threads are started."""
import time
from concurrent.futures import Future

import numpy as np

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
