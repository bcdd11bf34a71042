"""GPU: the continuous-batching engine returns the same result for a request
alone and in a concurrent mix, and respects its HBM admission budget."""
import numpy as np
import pytest

from qvm_gb300 import circuits
from qvm_gb300.serve import Request, Server
from qvm_gb300.state import state_bytes

pytestmark = pytest.mark.gpu


def _requests():
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(24):
        n = int(rng.integers(10, 21))
        fam = i % 3
        if fam == 0:
            gates = circuits.random_layers(n, layers=int(rng.integers(2, 8)), seed=i)
        elif fam == 1:
            gates = circuits.qft(n)
        else:
            m = n - (n % 2)
            e = circuits.random_3_regular_graph(m, rng)
            gates = circuits.qaoa_maxcut(m, e, [0.4, 0.9], [0.3, 0.2])
        prec = "fp32" if i % 2 else "fp64"
        shots = int(rng.integers(1, 2000))
        reqs.append(Request(n, gates, shots, prec, rng.random(shots), True, f"r{i}"))
    return reqs


def test_same_result_alone_and_in_mix(gpu):
    reqs = _requests()
    alone = {}
    srv = Server(hbm_budget=8e9, workers=1, fast_workers=0)
    for r in reqs:
        alone[r.tag] = srv.submit(r).result().shots
    srv.close()
    # the mix: many workers, a tight budget that forces admission waits
    budget = max(state_bytes(r.n, r.precision) for r in reqs) * 3
    srv = Server(hbm_budget=budget, workers=8)
    futs = [(r.tag, srv.submit(r)) for r in reqs]
    for tag, f in futs:
        np.testing.assert_array_equal(f.result().shots, alone[tag])
        assert srv.reserved <= budget
    srv.close()


def test_oversized_request_rejected(gpu):
    srv = Server(hbm_budget=1e6, workers=1)
    with pytest.raises(ValueError):
        srv.submit(Request(20, circuits.qft(20), 1, "fp64"))
    srv.close()


def test_priority_classes_give_identical_results(gpu):
    """qvmg_state_set_priority changes the stream priority and, for -1, the
    tile-pass grid (short CTAs); the amplitudes are bit-identical."""
    n = 20
    gs = circuits.random_su_circuit(n, depth=6, seed=4)
    from qvm_gb300 import CudaPureState, Program
    p = Program()
    p.add_gates(gs)
    p.plan(n, "fp32", fused=True, fusion_width=2, tile_qubits=12)
    out = {}
    for prio in (0, -1, 1, 0):
        s = CudaPureState(n, "fp32")
        s.set_priority(prio)
        p.run(s, fused=True)
        out.setdefault(prio, []).append(s.state_elements())
        s.free()
    ref = out[0][0]
    for prio, states in out.items():
        for st in states:
            np.testing.assert_array_equal(st, ref)
    with pytest.raises(Exception):
        s = CudaPureState(4, "fp32")
        try:
            s.set_priority(2)
        finally:
            s.free()


def test_device_reserve_and_out_of_memory(gpu):
    """qvmg_device_reserve maps pool memory once; a reservation beyond the
    device returns QVMG_E_NOMEM and keeps nothing (the pool's unused memory
    goes back to the device), and states still allocate and compute
    afterwards."""
    from qvm_gb300 import CudaPureState, _lib as L
    assert L.lib().qvmg_device_reserve(1 << 30) == 0
    assert L.lib().qvmg_device_reserve(1 << 50) == 3  # QVMG_E_NOMEM
    s = CudaPureState(26, "fp64")
    try:
        from qvm_gb300 import gates as G
        s.apply_matrix(G.gate_matrix("H"), [25])
        assert abs(s.excited_probability(25) - 0.5) < 1e-12
        assert abs(s.norm() - 1.0) < 1e-12
    finally:
        s.free()
