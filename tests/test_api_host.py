"""Host-side logic of the server endpoints (no GPU): address queries, qubit
relabeling, the terminal-measurement test that picks multishot's fast path,
result collection and the draw-stream rewind."""
import random

from qvm_gb300 import api
from qvm_gb300 import quil as Q
from qvm_gb300.state import Program


def test_valid_address_query():
    assert api.valid_address_query({"ro": True, "b": [0, 3], "c": None, "d": []})
    assert not api.valid_address_query({"ro": [-1]})
    assert not api.valid_address_query({"ro": [1.5]})
    assert not api.valid_address_query({1: True})
    assert not api.valid_address_query([("ro", True)])
    assert not api.valid_address_query({"ro": False})


def test_relabel():
    # app/src/api/multishot-measure.lisp:61-75: position in the relabeling
    assert api.relabel([0, 5, 2], 3, [2, 0, 7]) == ([1, api.UNUSED, 0], 3)
    assert api.relabel([7], 1, [2, 0, 7]) == ([2], 3)
    assert api.relabel([9], 2, [2, 0, 7]) == ([api.UNUSED], 2)
    assert api.relabel([1, 2], 4, None) == ([1, 2], 4)


def test_collect_like_reference():
    results = {"ro": [], "x": [], "y": []}
    mem = {"ro": [1, 0, 1], "x": [0, 1], "y": [1]}
    api._collect(mem, {"ro": True, "x": [1, 0], "y": None}, results)
    api._collect(mem, {"ro": True, "x": [1, 0], "y": None}, results)
    assert results == {"ro": [[1, 0, 1]] * 2, "x": [[1, 0]] * 2, "y": [[]] * 2}


def test_terminal_measurements():
    p = Program()
    m0, m1 = Q.Measure(0, ("ro", 0)), Q.Measure(1, None)
    assert api._terminal_measurements([p, p, m0, m1]) == ([p, p], [m0, m1])
    assert api._terminal_measurements([m0]) == ([], [m0])
    assert api._terminal_measurements([p]) == ([p], [])
    assert api._terminal_measurements([p, m0, p]) is None          # gate after a measurement
    assert api._terminal_measurements([p, Q.Reset(), m0]) is None  # RESET
    ma = Q.MeasureAll([(0, ("ro", 0))])
    assert api._terminal_measurements([p, ma]) == ([p], [ma])
    assert api._terminal_measurements([p, ma, m0]) is None         # mixed kinds
    p.free()


def test_segments_of_parsed_program():
    """The QVM groups gates into programs; terminal measures stay separate."""
    prog = Q.parse("DECLARE ro BIT[2]\nH 0\nCNOT 0 1\nMEASURE 0 ro[0]\nMEASURE 1 ro[1]")
    ins = prog.instructions
    assert [type(i).__name__ for i in ins] == ["GateApp", "GateApp", "Measure", "Measure"]
    chains = Q.compile_measure_chains(ins, 2)
    assert isinstance(chains[-1], Q.MeasureAll)
    assert chains[-1].storage == [(0, ("ro", 0)), (1, ("ro", 1))]


def test_take_draws_rewind():
    r = random.Random(3)
    draws, rewind = api._take_draws(r, 10)
    rewind(4)
    ref = random.Random(3)
    seq = [ref.random() for _ in range(10)]
    assert draws == seq
    ref2 = random.Random(3)
    for _ in range(4):
        ref2.random()
    assert r.random() == ref2.random()
