"""GPU parity of the batched QAOA engine against the CPU oracle."""
import os

import numpy as np
import pytest

from qvm_gb300 import circuits
from qvm_gb300.batch import QaoaBatch, random_qaoa_batch

pytestmark = pytest.mark.gpu


def oracle_qaoa(oracle, n, edges, gammas, betas):
    wf = oracle.zero_state(n)
    for m, qs in circuits.qaoa_maxcut(n, edges, gammas, betas):
        oracle.apply_matrix_operator(wf, m, qs)
    return wf


def test_qaoa_batch_matches_oracle(gpu, oracle):
    # sizes cover the shared-memory path (<= 13 qubits) and the HBM path
    graphs, gam, bet = random_qaoa_batch(10, [4, 6, 8, 12, 14, 16], 2, p=3, seed=1)
    b = QaoaBatch(graphs, gam, bet)
    nshots = 256
    draws = np.random.default_rng(2).random((len(graphs), nshots))
    ex, shots = b.run(draws)
    for i, (n, edges) in enumerate(graphs):
        want = oracle_qaoa(oracle, n, edges, gam[i], bet[i])
        got = b.state(i)
        assert np.max(np.abs(got - want)) < 2e-6, (i, n)
        cut = circuits.maxcut_values(n, edges)
        wex = float(np.sum(np.abs(want) ** 2 * cut))
        assert abs(ex[i] - wex) < 1e-5 * max(1.0, wex), (i, ex[i], wex)
        # shots: smallest x with C(x) >= draw on the renormalised FP32 state
        ref = got.astype(np.complex64).astype(np.complex128)
        tot = np.sum(np.abs(ref) ** 2)
        wsh = oracle.sample_multiple(ref, draws[i] * tot)
        cdf = np.cumsum(np.abs(ref) ** 2)
        near = np.array([np.min(np.abs(cdf - d * tot)) < 1e-9 for d in draws[i]])
        assert ((shots[i] == wsh) | near).all(), (i, n)
    b.free()


def test_qaoa_batch_rerun_and_new_angles(gpu):
    graphs, gam, bet = random_qaoa_batch(6, [12, 14, 18], 2, p=4, seed=3)
    b = QaoaBatch(graphs, gam, bet)
    e1, _ = b.run()
    e2, _ = b.run()
    np.testing.assert_array_equal(e1, e2)  # deterministic replay of the graph
    b.set_angles(gam * 0.5, bet * 0.5)
    e3, _ = b.run()
    assert not np.allclose(e1, e3)
    b.free()


def test_qaoa_batch_cut_paths(gpu, oracle):
    """The kernel splits each amplitude's cut into a low-bit table, a high-bit
    constant and popcounts over cross-edge slots (at most 4 cross edges per
    low qubit); a graph with more falls back to the edge loop.  Against the
    oracle: split path -- qubit 0 with three cross edges (slots 0-2) beside
    low-low and high-high edges (hub, 16 qubits), several low qubits with one
    cross edge each (fan), a 15-qubit mix; fallback -- qubit 0 with five cross
    edges (over, 18 qubits)."""
    hub = (16, [(0, 13), (0, 14), (0, 15), (0, 12), (1, 13), (2, 3), (4, 14), (5, 15),
                (13, 15), (6, 7), (0, 5)])
    fan = (16, [(0, 13), (0, 14), (0, 15)] + [(1, 13), (2, 14), (3, 15)] + [(0, 12)])
    mixed = (15, [(0, 13), (0, 14), (1, 13), (2, 14), (1, 2), (13, 14), (3, 12), (12, 13),
                  (5, 6), (0, 5)])
    # qubit 0 with 5 cross edges: n = 18 gives high qubits 13..17
    over = (18, [(0, 13), (0, 14), (0, 15), (0, 16), (0, 17), (1, 2), (13, 17), (3, 16)])
    graphs = [hub, fan, mixed, over]
    rng = np.random.default_rng(5)
    gam = [rng.uniform(0, np.pi, 2) for _ in graphs]
    bet = [rng.uniform(0, np.pi / 2, 2) for _ in graphs]
    b = QaoaBatch(graphs, gam, bet)
    ex, _ = b.run(np.random.default_rng(6).random((len(graphs), 4)))
    for i, (n, edges) in enumerate(graphs):
        want = oracle_qaoa(oracle, n, edges, gam[i], bet[i])
        assert np.max(np.abs(b.state(i) - want)) < 2e-6, (i, n)
        wex = float(np.sum(np.abs(want) ** 2 * circuits.maxcut_values(n, edges)))
        assert abs(ex[i] - wex) < 1e-5 * max(1.0, wex), (i, ex[i], wex)
    b.free()


def test_qaoa_batch_full_size_instances_match_oracle(gpu, oracle):
    """The workload's largest instances (n = 18, 20, 22) beside small ones,
    against the oracle: amplitudes, <H_C> and 1024 shots per instance."""
    oracle.set_workers(os.cpu_count() or 1)
    graphs, gam, bet = random_qaoa_batch(5, [12, 18, 20, 22], 1, p=4, seed=9)
    rng = np.random.default_rng(10)
    big = [(n, circuits.random_3_regular_graph(n, rng)) for n in (18, 20, 22)]
    graphs = big + graphs
    gam = np.vstack([rng.uniform(0, np.pi, (3, 4)), gam])
    bet = np.vstack([rng.uniform(0, np.pi / 2, (3, 4)), bet])
    b = QaoaBatch(graphs, gam, bet)
    draws = np.random.default_rng(11).random((len(graphs), 1024))
    ex, shots = b.run(draws)
    for i, (n, edges) in enumerate(graphs):
        want = oracle_qaoa(oracle, n, edges, gam[i], bet[i])
        got = b.state(i)
        assert np.max(np.abs(got - want)) < 2e-6, (i, n)
        wex = float(np.sum(np.abs(want) ** 2 * circuits.maxcut_values(n, edges)))
        assert abs(ex[i] - wex) < 1e-5 * max(1.0, wex), (i, ex[i], wex)
        ref = got.astype(np.complex64).astype(np.complex128)
        tot = np.sum(np.abs(ref) ** 2)
        wsh = oracle.sample_multiple(ref, draws[i] * tot)
        cdf = np.cumsum(np.abs(ref) ** 2)
        near = np.array([np.min(np.abs(cdf - d * tot)) < 1e-9 for d in draws[i]])
        assert ((shots[i] == wsh) | near).all(), (i, n)
    b.free()


def test_qaoa_batch_shot_buffer_failure_leaves_batch_usable(gpu):
    """Growing the shot buffers fails on its second allocation (made to fail
    on the host through the library's test hook): the run reports
    QVMG_E_NOMEM, and the batch then runs correctly with that shot count and
    with the old one (no cached graph keeps the freed buffers)."""
    from qvm_gb300 import QVMGError
    from qvm_gb300 import _lib as L
    graphs, gam, bet = random_qaoa_batch(3, [8, 12], 1, p=2, seed=7)
    b = QaoaBatch(graphs, gam, bet)
    rng = np.random.default_rng(3)
    d4, d64 = rng.random((len(graphs), 4)), rng.random((len(graphs), 64))
    e4, s4 = b.run(d4)
    L.call("qvmg_debug_fail_alloc", 2)
    try:
        with pytest.raises(QVMGError, match="batch draws and shots") as err:
            b.run(d64)
        assert err.value.code == 3  # QVMG_E_NOMEM
    finally:
        L.call("qvmg_debug_fail_alloc", 0)
    e4b, s4b = b.run(d4)
    e64, s64 = b.run(d64)
    fresh = QaoaBatch(graphs, gam, bet)
    fe64, fs64 = fresh.run(d64)
    np.testing.assert_array_equal(e4, e4b)
    np.testing.assert_array_equal(s4, s4b)
    np.testing.assert_array_equal(e64, fe64)
    np.testing.assert_array_equal(s64, fs64)
    b.free()
    fresh.free()


def test_qaoa_batch_wide_instances_match_oracle(gpu, oracle):
    """Instances of 23-26 qubits, whose row passes hold rows of 8, 2, 4 and
    1 amplitudes (their cut bytes then load one by one): depth 1 ends on a
    row pass, so <H_C> and the CDF are read back from HBM; depth 2 ends on a
    contiguous pass, which sums them from its tiles.  Against the oracle:
    amplitudes, <H_C> and 256 shots per instance."""
    oracle.set_workers(os.cpu_count() or 1)
    rng = np.random.default_rng(21)

    def ring_with_chords(n, chords):
        e = [(i, (i + 1) % n) for i in range(n)]
        while len(e) < n + chords:
            u, v = (int(x) for x in rng.choice(n, 2, replace=False))
            if (u, v) not in e and (v, u) not in e:
                e.append((u, v))
        return e

    cases = ((1, [(23, ring_with_chords(23, 10)), (26, circuits.random_3_regular_graph(26, rng))]),
             (2, [(24, circuits.random_3_regular_graph(24, rng)), (25, ring_with_chords(25, 8))]))
    for p, graphs in cases:
        gam = rng.uniform(0, np.pi, (len(graphs), p))
        bet = rng.uniform(0, np.pi / 2, (len(graphs), p))
        b = QaoaBatch(graphs, gam, bet)
        draws = np.random.default_rng(22).random((len(graphs), 256))
        ex, shots = b.run(draws)
        for i, (n, edges) in enumerate(graphs):
            want = oracle_qaoa(oracle, n, edges, gam[i], bet[i])
            got = b.state(i)
            assert np.max(np.abs(got - want)) < 2e-6, (p, n)
            wex = float(np.sum(np.abs(want) ** 2 * circuits.maxcut_values(n, edges)))
            assert abs(ex[i] - wex) < 1e-5 * max(1.0, wex), (p, n, ex[i], wex)
            ref = got.astype(np.complex64).astype(np.complex128)
            tot = np.sum(np.abs(ref) ** 2)
            wsh = oracle.sample_multiple(ref, draws[i] * tot)
            cdf = np.cumsum(np.abs(ref) ** 2)
            near = np.array([np.min(np.abs(cdf - d * tot)) < 1e-9 for d in draws[i]])
            assert ((shots[i] == wsh) | near).all(), (p, n)
        b.free()


@pytest.mark.parametrize("p", [7, 8])
def test_qaoa_batch_deep_circuits_match_oracle(gpu, oracle, p):
    """Depths 7 and 8: the p + 1 tile passes of an instance in HBM alternate
    between contiguous tiles and high-qubit rows p + 1 times, each finishing
    one layer's RX and starting the next; an odd depth ends on a row pass (the
    CDF and <H_C> read back from HBM), an even one on a contiguous pass (both
    summed from the tiles).  Beside them, instances that stay in shared
    memory.  Against the oracle: amplitudes, <H_C> and 256 shots each."""
    oracle.set_workers(os.cpu_count() or 1)
    rng = np.random.default_rng(40 + p)
    graphs = [(n, circuits.random_3_regular_graph(n, rng)) for n in (10, 16, 20, 14)]
    gam = rng.uniform(0, np.pi, (len(graphs), p))
    bet = rng.uniform(0, np.pi / 2, (len(graphs), p))
    b = QaoaBatch(graphs, gam, bet)
    draws = np.random.default_rng(50 + p).random((len(graphs), 256))
    ex, shots = b.run(draws)
    for i, (n, edges) in enumerate(graphs):
        want = oracle_qaoa(oracle, n, edges, gam[i], bet[i])
        got = b.state(i)
        assert np.max(np.abs(got - want)) < 4e-6, (p, n)
        wex = float(np.sum(np.abs(want) ** 2 * circuits.maxcut_values(n, edges)))
        assert abs(ex[i] - wex) < 1e-5 * max(1.0, wex), (p, n, ex[i], wex)
        ref = got.astype(np.complex64).astype(np.complex128)
        tot = np.sum(np.abs(ref) ** 2)
        wsh = oracle.sample_multiple(ref, draws[i] * tot)
        cdf = np.cumsum(np.abs(ref) ** 2)
        near = np.array([np.min(np.abs(cdf - d * tot)) < 1e-9 for d in draws[i]])
        assert ((shots[i] == wsh) | near).all(), (p, n)
    b.free()
