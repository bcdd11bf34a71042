"""Generate the full-size oracle fixtures (run once on a CPU host; minutes).

    python tests/golden/make_fullsize.py [qft28] [random30] [--threads T]

- ``qft28_fp64.npz``: the 28-qubit QFT (28 H, 378 CPHASE, 14 SWAP in the
  order of examples/qft.lisp) applied by the oracle's apply-matrix-operator
  to the seeded complex-Gaussian state ``circuits.random_state(28, seed=2)``.
- ``random30_layer1.npz``: the first full layer (30 Haar SU(2) + 15 Haar
  SU(4) on a random perfect matching) of the 30-qubit depth-20 random
  circuit ``circuits.random_su_circuit(30, 20, seed=3)`` applied to
  |0...0>, its gate matrices, 4096 uniform draws, the oracle's CDF samples
  for them (src/measurement.lisp:246-288) and the draws exempt from exact
  agreement (within 1e-12 plus the serial CDF's measured rounding of a
  boundary).

Each fixture holds the fingerprint of ``tests/fullsize_common.py``.  The
oracle runs with OpenMP on every host core.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from qvm_gb300 import circuits  # noqa: E402
from tests import fullsize_common as F  # noqa: E402


def _log(msg):
    print(time.strftime("%H:%M:%S"), msg, flush=True)


def make_qft28(path):
    n = 28
    wf = circuits.random_state(n, seed=2)
    gates = circuits.qft(n)
    t = time.time()
    for g, (m, qs) in enumerate(gates):
        O.apply_matrix_operator(wf, m, qs)
        if g % 20 == 0:
            _log(f"qft28 gate {g}/{len(gates)} ({time.time() - t:.0f} s)")
    fp = F.fingerprint(wf, n)
    np.savez_compressed(path, n=n, state_seed=2, norm=np.linalg.norm(wf), **fp)
    _log(f"wrote {path}")


def make_random30(path):
    n = 30
    layer = circuits.random_su_circuit(n, depth=20, seed=3)[:n + n // 2]
    wf = O.zero_state(n)
    t = time.time()
    for g, (m, qs) in enumerate(layer):
        O.apply_matrix_operator(wf, m, qs)
        _log(f"random30 gate {g}/{len(layer)} ({time.time() - t:.0f} s)")
    fp = F.fingerprint(wf, n)
    draws = np.random.default_rng(4).random(4096)
    shots = O.sample_multiple(wf, draws)
    _log("samples done")
    cdf = O.cdf(wf)
    exempt = F.cdf_boundary_exemptions(wf, draws, shots, cdf)
    del cdf
    _log(f"{int(exempt.sum())} of {len(draws)} draws exempt")
    mats = np.concatenate([np.asarray(m, dtype=np.complex128).ravel() for m, _ in layer])
    kq = np.array([len(qs) for _, qs in layer], dtype=np.int32)
    qubits = np.concatenate([np.asarray(qs, dtype=np.int32) for _, qs in layer])
    np.savez_compressed(path, n=n, circuit_seed=3, mats=mats, kq=kq, qubits=qubits,
                        draws=draws, shots=shots, exempt=exempt, **fp)
    _log(f"wrote {path}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="*", default=["qft28", "random30"])
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    a = ap.parse_args()
    O.build()
    O.set_workers(a.threads)
    if "random30" in a.which:
        make_random30(os.path.join(HERE, "random30_layer1.npz"))
    if "qft28" in a.which:
        make_qft28(os.path.join(HERE, "qft28_fp64.npz"))


if __name__ == "__main__":
    main()
