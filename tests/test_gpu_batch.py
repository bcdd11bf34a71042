"""GPU parity of the batched QAOA engine against the CPU oracle."""
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
