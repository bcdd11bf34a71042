"""The density-matrix op construction on the CPU: the 2n-qubit ops that
DensityQVM hands to the engine, executed by the oracle on vec(rho), equal
U rho U^H, sum_j K_j rho K_j^H, the measurement collapse and the dephasing
computed with numpy matrices."""
import numpy as np

from qvm_gb300 import gates
from qvm_gb300 import density as D
from qvm_gb300.noisy import make_pauli_perturbed_1q_gate


def random_rho(n, rng):
    a = rng.standard_normal((1 << n, 3)) + 1j * rng.standard_normal((1 << n, 3))
    rho = a @ a.conj().T
    return rho / np.trace(rho).real


def embed(m, nat_qubits, n):
    """Full 2^n matrix of a gate on nat-ordered qubits."""
    dim = 1 << n
    full = np.zeros((dim, dim), dtype=np.complex128)
    k = len(nat_qubits)
    for col in range(dim):
        c = sum(((col >> q) & 1) << j for j, q in enumerate(nat_qubits))
        for r in range(1 << k):
            row = col
            for j, q in enumerate(nat_qubits):
                row = (row & ~(1 << q)) | (((r >> j) & 1) << q)
            full[row, col] += m[r, c]
    return full


def run_ops(oracle, ops, vec):
    for kind, data, qs in ops:
        if kind == "perm":
            oracle.apply_permutation(vec, data, qs)
        elif kind == "diag":
            oracle.apply_matrix_operator(vec, np.diag(data), qs)
        else:
            oracle.apply_matrix_operator(vec, data, qs)
    return vec


def test_gate_ops(oracle):
    rng = np.random.default_rng(1)
    n = 3
    for k in (1, 2, 3):
        for _ in range(3):
            rho = random_rho(n, rng)
            u = gates.haar_unitary(rng, 1 << k)
            qs = [int(x) for x in rng.permutation(n)[:k]]
            got = run_ops(oracle, D.gate_ops(u, qs, n), rho.reshape(-1).copy())
            full = embed(u, qs, n)
            np.testing.assert_allclose(got.reshape(rho.shape), full @ rho @ full.conj().T,
                                       atol=1e-13)
    perm = [1, 0, 3, 2]
    qs = [2, 0]
    rho = random_rho(n, rng)
    got = run_ops(oracle, D.gate_ops(None, qs, n, perm=perm), rho.reshape(-1).copy())
    p = gates.permutation_matrix(perm)
    full = embed(p, qs, n)
    np.testing.assert_allclose(got.reshape(rho.shape), full @ rho @ full.T, atol=1e-14)


def test_kraus_superoperator(oracle):
    rng = np.random.default_rng(2)
    n = 3
    for qs, ops in (([1], make_pauli_perturbed_1q_gate("H", 0.1, 0.2, 0.05)),
                    ([2, 0], [np.sqrt(0.7) * gates.haar_unitary(rng, 4),
                              np.sqrt(0.3) * gates.haar_unitary(rng, 4)])):
        rho = random_rho(n, rng)
        got = run_ops(oracle, D.kraus_ops_on_density(ops, qs, n), rho.reshape(-1).copy())
        want = sum(embed(k, qs, n) @ rho @ embed(k, qs, n).conj().T for k in ops)
        np.testing.assert_allclose(got.reshape(rho.shape), want, atol=1e-13)


def test_collapse_and_dephase(oracle):
    rng = np.random.default_rng(3)
    n = 3
    rho = random_rho(n, rng)
    q = 1
    idx = np.arange(1 << n)
    p1 = float(np.sum(np.diag(rho).real[(idx >> q) & 1 == 1]))
    for bit in (0, 1):
        got = run_ops(oracle, [("diag", D.collapse_diagonal(bit, p1), [q, q + n])],
                      rho.reshape(-1).copy()).reshape(rho.shape)
        proj = np.diag(((idx >> q) & 1 == bit).astype(float))
        want = proj @ rho @ proj / (p1 if bit else 1 - p1)
        np.testing.assert_allclose(got, want, atol=1e-14)
        assert abs(np.trace(got).real - 1) < 1e-13
    got = run_ops(oracle, [("diag", D.DEPHASE, [q, q + n])], rho.reshape(-1).copy())
    keep = ((idx[:, None] >> q) & 1) == ((idx[None, :] >> q) & 1)
    np.testing.assert_allclose(got.reshape(rho.shape), np.where(keep, rho, 0), atol=0)
