"""Autotuner for the fused path: fusion width, tile width and tile engine.

For a program and a state size it plans and runs every candidate
(fusion width, tile qubits, engine) once on the device, times the runs with
the per-pass CUDA events of ``Program.run_profiled``, and keeps the fastest.
Engines of an FP32 tile: "fma" (every block through shared memory on FP32
FMAs), "reg" (runs of 1-/2-qubit blocks on amplitudes held in registers) and
"tc" (blocks merged to 3-5 qubits and run as tcgen05 bf16x3 MMAs).
Results are cached on the Program object itself, per (qubits, precision,
candidate list, op-list generation): a freed program's choice can never be
served to a new one, and adding ops to a program retunes it.
"""
from __future__ import annotations

import numpy as np

from .state import CudaPureState, Program

ENGINES = ("fma", "reg", "tc")

DEFAULT_CANDIDATES = {
    "fp32": [(fw, t, e) for fw in (1, 2) for t in (12, 13, 14) for e in ("fma", "reg")
             if not (e == "reg" and t == 14)] + [(4, 12, "tc"), (4, 13, "tc"), (5, 13, "tc"),
                                                   (2, 13, "tc")],
    "fp64": [(fw, t, "fma") for fw in (1, 2, 3) for t in (11, 12, 13)],
}


def apply_engine(prog: Program, engine: str):
    prog.set_register_stages(engine == "reg")
    prog.set_tensor_cores(engine == "tc")


def autotune(prog: Program, state: CudaPureState, precision: str = "fp32", candidates=None,
             repeats: int = 1):
    """Pick (fusion_width, tile_qubits, engine) for `prog` on `state`;
    returns (best, table) with table[candidate] = device ms per run.  The
    state is overwritten (it is reset before every trial)."""
    n = state.num_qubits()
    cands = tuple(candidates or DEFAULT_CANDIDATES[precision])
    cache = prog.__dict__.setdefault("_autotune_cache", {})
    key = (n, precision, cands, prog.generation)
    if key in cache:
        choice, table = cache[key]
        apply_engine(prog, choice[2])
        prog.plan(n, precision, fused=True, fusion_width=choice[0], tile_qubits=choice[1])
        return choice, table
    table = {}
    for fw, tile, engine in cands:
        try:
            apply_engine(prog, engine)
            prog.plan(n, precision, fused=True, fusion_width=fw, tile_qubits=tile)
        except Exception:
            continue
        best = np.inf
        for _ in range(repeats + 1):        # first run uploads the plan
            state.set_to_zero_state()
            ms, _ = prog.run_profiled(state, fused=True)
            best = min(best, float(ms.sum()))
        table[(fw, tile, engine)] = best
    choice = min(table, key=table.get)
    apply_engine(prog, choice[2])
    prog.plan(n, precision, fused=True, fusion_width=choice[0], tile_qubits=choice[1])
    cache[key] = (choice, table)
    return choice, table
