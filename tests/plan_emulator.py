"""Execute a plan description (qvmg_program_plan_describe) on the CPU with the
oracle, to check the planner's fusion and tiling logic without a GPU.

Test infrastructure: the library itself never executes plans on the CPU.
"""
import numpy as np


def _cplx(pairs):
    a = np.array(pairs, dtype=np.float64).reshape(-1, 2)
    return a[:, 0] + 1j * a[:, 1]


def _apply_table(wf, qubits, table):
    idx = np.arange(len(wf), dtype=np.int64)
    sub = np.zeros(len(wf), dtype=np.int64)
    for j, q in enumerate(qubits):
        sub |= ((idx >> q) & 1) << j
    wf *= table[sub]


def tc_matrix(pairs, k):
    """The complex block of a tensor-core tile op from its operand: the bf16
    hi + lo parts of the real form Bt (n = 2r + re/im of output r,
    kk = 2c + re/im of input c), K-major 8x8 core matrices, carried as the
    bit patterns of FP32 values (two bf16 per float, low half first)."""
    f = np.array(pairs, dtype=np.float64).reshape(-1).astype(np.float32)
    h = f.view(np.uint32)
    u16 = np.empty(2 * len(h), dtype=np.uint32)
    u16[0::2] = h & 0xFFFF
    u16[1::2] = h >> 16
    vals = (u16 << 16).astype(np.uint32).view(np.float32).astype(np.float64)
    d = 1 << k
    nk = 2 * d
    n = np.arange(nk)[:, None]
    kk = np.arange(nk)[None, :]
    idx = ((n >> 3) * (nk >> 3) + (kk >> 3)) * 64 + (n & 7) * 8 + (kk & 7)
    bt = vals[idx] + vals[nk * nk + idx]
    re, im = bt[0::2, 0::2], bt[1::2, 0::2]
    assert np.array_equal(bt[1::2, 1::2], re) and np.array_equal(bt[0::2, 1::2], -im)
    return re + 1j * im


def run_description(oracle, desc, wf):
    for p in desc["passes"]:
        kind = p["kind"]
        if kind == "dense":
            d = 1 << len(p["qubits"])
            oracle.apply_matrix_operator(wf, _cplx(p["matrix"]).reshape(d, d), p["qubits"])
        elif kind == "perm":
            oracle.apply_permutation(wf, p["perm"], p["qubits"])
        elif kind == "diag":
            for t in p["tables"]:
                _apply_table(wf, t["qubits"], _cplx(t["table"]))
        else:
            L, E = p["L"], p["E"]
            glob = lambda pos: pos if pos < L else E[pos - L]  # noqa: E731
            for op in p["ops"]:
                if op["kind"] == "diag":
                    _apply_table(wf, op["pos"], _cplx(op["data"]))
                elif op["kind"] == "perm":
                    oracle.apply_permutation(wf, op["perm"], [glob(x) for x in op["pos"]])
                elif op["kind"] == "tc":
                    m = tc_matrix(op["data"], len(op["pos"]))
                    oracle.apply_matrix_operator(wf, m, [glob(x) for x in op["pos"]])
                else:
                    k = len(op["pos"])
                    m = _cplx(op["data"]).reshape(1 << k, 1 << k)
                    oracle.apply_matrix_operator(wf, m, [glob(x) for x in op["pos"]])
    return wf
