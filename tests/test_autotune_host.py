"""The autotuner's choice and cache, with a fake program and state (no GPU):
the choice is the timing table's minimum, each program keeps its own
entry, and adding ops to a program retunes it."""
import numpy as np

from qvm_gb300 import autotune as A


class _FakeState:
    def __init__(self, n):
        self.n = n
        self.resets = 0

    def num_qubits(self):
        return self.n

    def set_to_zero_state(self):
        self.resets += 1


class _FakeProgram:
    """Device time of a run = cost[(fw, tile, engine)]; plans that the table
    marks None raise, as an over-budget plan does."""

    def __init__(self, cost):
        self.cost = dict(cost)
        self.generation = 0
        self.engine = {"reg": False, "tc": False}
        self.planned = None
        self.runs = 0

    def set_register_stages(self, on):
        self.engine["reg"] = on

    def set_tensor_cores(self, on):
        self.engine["tc"] = on

    def _engine(self):
        return "reg" if self.engine["reg"] else ("tc" if self.engine["tc"] else "fma")

    def plan(self, n, precision, fused=True, fusion_width=2, tile_qubits=0):
        key = (fusion_width, tile_qubits, self._engine())
        if self.cost.get(key) is None:
            raise RuntimeError("plan over budget")
        self.planned = key

    def run_profiled(self, state, fused=True):
        self.runs += 1
        return np.array([self.cost[self.planned] / 2] * 2), np.array([3, 3])

    def add_gates(self, gates):
        self.generation += 1


CANDS = [(1, 12, "fma"), (2, 13, "fma"), (2, 13, "reg"), (4, 13, "tc"), (2, 14, "fma")]


def test_choice_is_table_minimum_and_cache_is_per_program():
    cost_a = {(1, 12, "fma"): 9.0, (2, 13, "fma"): 5.0, (2, 13, "reg"): 7.0,
              (4, 13, "tc"): 4.0, (2, 14, "fma"): None}
    cost_b = dict(cost_a)
    cost_b[(4, 13, "tc")] = 8.0
    pa, pb = _FakeProgram(cost_a), _FakeProgram(cost_b)
    st = _FakeState(20)
    choice, table = A.autotune(pa, st, "fp32", candidates=CANDS)
    assert choice == min(table, key=table.get) == (4, 13, "tc")
    assert (2, 14, "fma") not in table            # the failing plan is skipped
    assert pa.planned == choice                   # left planned with the choice
    runs = pa.runs
    # cached: no new trial runs, and the choice is re-applied
    pa.planned = None
    assert A.autotune(pa, st, "fp32", candidates=CANDS)[0] == choice
    assert pa.runs == runs and pa.planned == choice
    # a different program is tuned on its own timings
    cb, tb = A.autotune(pb, st, "fp32", candidates=CANDS)
    assert cb == (2, 13, "fma") == min(tb, key=tb.get)


def test_added_ops_retune():
    cost = {(1, 12, "fma"): 3.0, (2, 13, "fma"): 5.0, (2, 13, "reg"): 7.0,
            (4, 13, "tc"): 4.0, (2, 14, "fma"): 6.0}
    p = _FakeProgram(cost)
    st = _FakeState(16)
    assert A.autotune(p, st, "fp32", candidates=CANDS)[0] == (1, 12, "fma")
    p.add_gates([None])
    p.cost[(1, 12, "fma")] = 10.0
    assert A.autotune(p, st, "fp32", candidates=CANDS)[0] == (4, 13, "tc")
