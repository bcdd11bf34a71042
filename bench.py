#!/usr/bin/env python
"""Benchmark: 30-qubit depth-20 random SU(2)/SU(4) circuit, gates/s.

One step = reset a 30-qubit state to |0...0> and run the whole 900-gate
circuit (per layer: a Haar SU(2) on every qubit, then a Haar SU(4) on each
pair of a random perfect matching; seeded synthetic input) through the fused
FP32 path, state resident in HBM.  The line also reports the plain FP64
kernels and the fused double-float FP64 tiles on the same circuit, the
fused-FP32 vs FP64 fidelity and max amplitude error, 4096 shots sampled from
both states with the same uniform draws, the tile kernel's roofline, an
end-to-end number through the public API with host buffers, a CPU baseline
(the oracle restatement of the reference's per-gate algorithm on the host
cores, FP64) and the precision-matched ratios against it, plus the other
workloads (32-qubit circuit, 28-qubit FP64 QFT, batched QAOA, serving, ...).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank runs an independent replica on its own GPU
(the workload does not shard); value = all ranks' gates / max rank time.
With --impl reference, one step is a fixed 15-gate sample of the circuit
(a third of a layer, the layer's gate mix) on the CPU port, FP64.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "30q gates/s fused-FP32 vs plain FP64 at fidelity>=1-1e-6; %HBM peak; p99 latency"
UNIT = "gates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=30)
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--shots", type=int, default=4096)
    ap.add_argument("--fw", type=int, default=0, help="fusion width (0: autotune)")
    ap.add_argument("--tile", type=int, default=0, help="tile qubits (0: autotune)")
    ap.add_argument("--engine", default="auto", choices=["auto", "fma", "reg", "tc"],
                    help="tile engine: FP32 FMAs, register stages or tcgen05 tensor cores "
                         "(auto: tune)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched QAOA run")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving stream")
    ap.add_argument("--no-qft", action="store_true", help="skip the 28-qubit FP64 QFT")
    ap.add_argument("--qft-n", type=int, default=28,
                    help="qubits of the FP64 QFT leg (smaller for profiling)")
    ap.add_argument("--no-32q", action="store_true", help="skip the 32-qubit random circuit")
    ap.add_argument("--no-endpoints", action="store_true",
                    help="skip the server-endpoint and noise measurements")
    ap.add_argument("--no-plain-passes", action="store_true",
                    help="skip the per-kind timing of memory-bound plain passes")
    ap.add_argument("--no-layers", action="store_true",
                    help="skip the 20-qubit layer circuit with 1000 shots")
    ap.add_argument("--cpu-steps", type=int, default=3,
                    help="timed samples of the CPU baseline (about 6 s each at 30 qubits)")
    ap.add_argument("--no-32q-plain", action="store_true",
                    help="skip the plain FP64 kernels at 32 qubits (about 80 s)")
    ap.add_argument("--case", default=None, choices=sorted(PROFILE_CASES),
                    help="run one small workload of a kernel family and exit (for ncu "
                         "captures; prints a one-line summary, not the bench line)")
    return ap.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float) -> float:
    """The slowest rank's time (all_reduce MAX; NCCL on GPUs, gloo on CPU)."""
    import torch
    import torch.distributed as tdist
    if not tdist.is_initialized() or tdist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if tdist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step: int, steps: int, world: int, max_ms: float) -> float:
    """Units all ranks processed divided by the slowest rank's time."""
    return world * units_per_rank_step * steps / (max_ms / 1e3)


# DRAM bytes (read + write) of one fused FP32 tile launch at 26 qubits, from
# the ncu captures summarised under profiles/ (k_tile_fp32_random26_fw2_t13,
# k_tile_tc_bf16x3_random26_fw5_t13).  Traffic per launch grows with the
# amplitudes processed, so a launch at n qubits moves 2^(n-26) times as much.
TILE_TRAFFIC_26Q = {"fma": 536.987648e6 + 475.479808e6, "tc": 536.993792e6 + 474.862848e6}


def traffic_per_launch(n, engine):
    b = TILE_TRAFFIC_26Q.get(engine)
    return None if b is None else b * 2.0 ** (n - 26)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def reference_sample(gates, n, j):
    """The j-th fixed CPU-timing sample of the circuit: one third of layer
    (j // 3) mod depth, part r = j % 3 -- that layer's SU(2)s on the r-th
    third of the qubits followed by the r-th third of its SU(4)s (for 30
    qubits 10 SU(2) + 5 SU(4), the same 2:1 mix as a whole layer), in circuit
    order.  Used by the reference arm and the CPU baseline alike."""
    per_layer = n + n // 2
    depth = len(gates) // per_layer
    layer = (j // 3) % depth
    r = j % 3
    base = layer * per_layer
    one = np.array_split(np.arange(n), 3)[r]
    two = np.array_split(np.arange(n // 2), 3)[r]
    return [gates[base + int(i)] for i in one] + [gates[base + n + int(i)] for i in two]


def cpu_baseline(n, gates, steps, threads):
    """The oracle (restatement of the reference's per-gate apply-matrix-
    operator with worker-parallel loops) on the host cores: one untimed
    sample, then `steps` timed samples of the circuit (reference_sample),
    applied in turn to one FP64 state."""
    from oracle import oracle as O
    O.set_workers(threads, threshold=19)
    wf = O.zero_state(n)
    for m, qs in reference_sample(gates, n, 0):
        O.apply_matrix_operator(wf, m, qs)
    done, dt = 0, 0.0
    for j in range(1, steps + 1):
        sample = reference_sample(gates, n, j)
        t0 = time.perf_counter()
        for m, qs in sample:
            O.apply_matrix_operator(wf, m, qs)
        dt += time.perf_counter() - t0
        done += len(sample)
    del wf
    return {"value": done / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} samples of {done // steps} gates (one third of a layer: "
                      f"{n // 3} SU(2) + {n // 6} SU(4)) of the {n}-qubit circuit, FP64, "
                      f"{dt:.1f} s"}


def run_qaoa_batch(seed: int = 4, runs: int = 3):
    """Batched QAOA MaxCut: 512 random 3-regular graphs with n in {12..22},
    8 (gamma, beta) sets each = 4096 instances, p = 4, 1024 shots each, one
    persistent launch per run (CUDA graph).  Timed end to end per run, with
    the draws' upload and the shots' and expectations' download."""
    from qvm_gb300.batch import QaoaBatch, random_qaoa_batch
    graphs, gam, bet = random_qaoa_batch(512, [12, 14, 16, 18, 20, 22], 8, p=4, seed=seed)
    b = QaoaBatch(graphs, gam, bet)
    draws = np.random.default_rng(seed).random((len(graphs), 1024))
    ex, shots = b.run(draws)  # warm-up (graph capture)
    times = []
    for _ in range(runs):
        t0 = time.perf_counter()
        ex, shots = b.run(draws)
        times.append(time.perf_counter() - t0)
    ngates = sum(n + 4 * (len(e) + n) for n, e in graphs)
    dt = float(np.median(times))
    out = {"instances": len(graphs), "qubits": "12..22", "p": 4, "shots_per_instance": 1024,
           "ms_per_batch": 1e3 * dt, "instances_per_s": len(graphs) / dt,
           "gates_per_s": ngates / dt, "device_gib": b.device_bytes() / 2 ** 30,
           "expectation_mean": float(np.mean(ex)),
           "h2d_bytes": int(draws.nbytes), "d2h_bytes": int(shots.nbytes + ex.nbytes)}
    b.free()
    return out


def run_qft_fp64(n: int = 28, seed: int = 2, runs: int = 3):
    """28-qubit QFT in complex FP64, plain kernels (one pass per H and SWAP,
    one phase-table pass per CPHASE chain) on a random normalised state of
    complex N(0,1) amplitudes.  Reports gates/s and HBM GB/s per pass kind,
    from CUDA events around every pass.  Algorithmic bytes per pass: a dense
    pass reads and writes every amplitude (2 * 16 * 2^n); a phase pass and a
    SWAP the half they change (2 * 16 * 2^(n-1))."""
    from qvm_gb300 import CudaPureState, Program, circuits
    gates = circuits.qft(n)
    rng = np.random.default_rng(seed)
    wf = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    wf /= np.linalg.norm(wf)
    s = CudaPureState(n, "fp64")
    s.set_state_elements(wf)
    wf0 = wf
    prog = Program()
    prog.add_gates(gates)
    st = prog.plan(n, "fp64", fused=False)
    prog.run(s, fused=False)  # untimed: uploads the plan
    s.sync()
    amp = 16 * (1 << n)
    # dense: every amplitude read and written; a CPHASE chain's phase pass: the
    # half with the target bit set (the others keep phase 1 and are not
    # visited); a SWAP: the half it moves
    bytes_of = {0: 2 * amp, 1: amp, 2: amp}
    names = {0: "dense", 1: "phase", 2: "swap"}
    best = None
    for _ in range(runs):
        ms, kinds = prog.run_profiled(s, fused=False)
        if best is None or ms.sum() < best[0].sum():
            best = (ms, kinds)
    ms, kinds = best
    peak, _ = peaks()
    per = {}
    for k in (0, 1, 2):
        sel = kinds == k
        if sel.any():
            t = float(ms[sel].sum())
            gbs = bytes_of[k] * int(sel.sum()) / (t / 1e3) / 1e9
            per[names[k]] = {"passes": int(sel.sum()), "ms": t, "GB_per_s": gbs,
                             "frac_of_measured_peak": gbs / peak}
    total = float(ms.sum())
    moved = sum(bytes_of[int(k)] for k in kinds)
    # the same circuit fused (tile passes in double-float, diagonal tables
    # read in place), compared with one plain application to the same input
    s.set_state_elements(wf0)
    prog.run(s, fused=False)
    plain_out = s.state_elements()
    fst = prog.plan(n, "fp64", fused=True, fusion_width=2)
    fbest = None
    for _ in range(runs):
        s.set_state_elements(wf0)
        fms, _ = prog.run_profiled(s, fused=True)
        fbest = fms.sum() if fbest is None else min(fbest, fms.sum())
    fdiff = float(np.max(np.abs(s.state_elements() - plain_out)))
    del plain_out, wf0
    s.free()
    prog.free()
    return {"workload": f"QFT, {n} qubits, complex FP64, plain kernels, random normalised state",
            "gates": len(gates), "passes": st["passes"], "ms": total,
            "gates_per_s": len(gates) / (total / 1e3),
            "hbm_GB_per_s": moved / (total / 1e3) / 1e9,
            "frac_of_measured_peak": moved / (total / 1e3) / 1e9 / peak, "per_pass_kind": per,
            "fused": {"passes": fst["passes"], "ms": float(fbest),
                      "gates_per_s": len(gates) / (float(fbest) / 1e3),
                      "max_abs_diff_vs_plain": fdiff}}


def run_plain_passes(runs: int = 5, seed: int = 9):
    """Memory-bound plain passes, one per kind, on an 8 GiB state: FP32 at 30
    qubits and FP64 at 29.  Each gate below is one pass, timed with CUDA events
    around every pass; algorithmic bytes count the amplitudes a pass reads and
    writes: a dense 1-/2-qubit gate and RZ every amplitude (2*b*N), CPHASE the
    quarter whose phase is not 1, X every amplitude, CNOT and SWAP the half they
    move."""
    from qvm_gb300 import CudaPureState, Program, circuits, gates as G
    rng = np.random.default_rng(seed)
    peak, _ = peaks()
    out = {}
    for prec, n in (("fp32", 30), ("fp64", 29)):
        b = 8 if prec == "fp32" else 16
        N = float(1 << n)
        # (label, matrix, nat-tuple qubits, bytes)
        seq = [("H q29" if n == 30 else "H q28", G.gate_matrix("H"), [n - 1], 2 * b * N),
               ("RZ q5", G.gate_matrix("RZ", 0.3), [5], 2 * b * N),
               ("H q0", G.gate_matrix("H"), [0], 2 * b * N),
               ("SU4 q3,q27", circuits.haar_special_unitary(rng, 4), [27, 3], 2 * b * N),
               ("CPHASE q2,q9", G.gate_matrix("CPHASE", 0.1), [9, 2], 2 * b * N / 4),
               ("X q7", G.gate_matrix("X"), [7], 2 * b * N),
               ("CNOT q28,q4" if n == 30 else "CNOT q27,q4", G.gate_matrix("CNOT"),
                [4, n - 2], b * N),
               ("SWAP q1,q20", G.gate_matrix("SWAP"), [20, 1], b * N)]
        prog = Program()
        prog.add_gates([(m, q) for _, m, q, _ in seq])
        prog.plan(n, prec, fused=False)
        s = CudaPureState(n, prec)
        prog.run(s, fused=False)
        best = None
        for _ in range(runs):
            ms, kinds = prog.run_profiled(s, fused=False)
            best = ms if best is None else np.minimum(best, ms)
        s.free()
        prog.free()
        if len(best) != len(seq):
            out[prec] = {"error": f"{len(best)} passes for {len(seq)} gates"}
            continue
        rows = {}
        for (label, _, _, by), t in zip(seq, best):
            gbs = by / (t / 1e3) / 1e9
            rows[label] = {"ms": float(t), "GB_per_s": gbs, "frac_of_measured_peak": gbs / peak}
        out[prec] = {"qubits": n, "passes": rows}
    return out


def run_engines_other(runs: int = 2):
    """The FP32 tile engines on circuits other than the headline: the layer
    circuit (H, then RX/RZ on every qubit and CNOTs on alternating pairs per
    layer) at 28 qubits with 10 layers, and the QFT at 30 qubits.  Each runs
    fused with the FMA engine (fusion width 2, 13-qubit tiles) and with the
    tensor-core engine (fusion width 5, 13-qubit tiles); device ms per run
    from per-pass events, plus the plan's tensor-core block count."""
    from qvm_gb300 import CudaPureState, Program, circuits
    from qvm_gb300.autotune import apply_engine
    out = {}
    for name, n, gates in (("layers28", 28, circuits.random_layers(28, layers=10, seed=1)),
                           ("qft30", 30, circuits.qft(30))):
        s = CudaPureState(n, "fp32")
        row = {"qubits": n, "gates": len(gates)}
        for engine, fw, tile in (("fma", 2, 13), ("tc", 5, 13)):
            p = Program()
            p.add_gates(gates)
            apply_engine(p, engine)
            st = p.plan(n, "fp32", fused=True, fusion_width=fw, tile_qubits=tile)
            best = float("inf")
            for _ in range(runs + 1):
                s.set_to_zero_state()
                ms, _ = p.run_profiled(s, fused=True)
                best = min(best, float(ms.sum()))
            row[engine] = {"ms": best, "passes": st["passes"], "fusion_width": fw,
                           "tile_qubits": tile}
            if engine == "tc":
                d = p.describe()
                row[engine]["tc_blocks"] = sum(1 for ps in d["passes"] if ps["kind"] == "tile"
                                               for op in ps["ops"] if op["kind"] == "tc")
            p.free()
        s.free()
        out[name] = row
    return out


def run_layers_shots(n: int = 20, layers: int = 10, shots: int = 1000, seed: int = 1, runs: int = 5):
    """The plain small case: 20-qubit FP64 state, H on all qubits, 10 layers of
    RX/RZ on every qubit and CNOTs on alternating pairs, then measure-all for
    1000 shots (bisection rule on the reloaded state).  Timed end to end per
    run from |0...0> to the downloaded shots."""
    from qvm_gb300 import CudaPureState, Program, circuits
    gates = circuits.random_layers(n, layers=layers, seed=seed)
    s = CudaPureState(n, "fp64")
    prog = Program()
    prog.add_gates(gates)
    draws = np.random.default_rng(seed).random(shots)
    times = []
    for i in range(runs + 1):
        t0 = time.perf_counter()
        s.set_to_zero_state()
        prog.run(s, fused=False)
        out = s.sample(draws, rule="bisect")
        t1 = time.perf_counter()
        if i:
            times.append(t1 - t0)
    dt = float(np.median(times))
    s.free()
    prog.free()
    return {"workload": f"{n}-qubit RX/RZ/CNOT layers ({len(gates)} gates), FP64 plain kernels, "
                        f"{shots} measure-all shots", "ms": 1e3 * dt,
            "gates_per_s": len(gates) / dt, "shots_per_s": shots / dt,
            "first_shots": [int(x) for x in out[:4]]}


def run_endpoints(n: int = 26, seed: int = 7):
    """The server endpoints and noise paths on a resident state, each against
    the reference's own algorithm run on the same GPU where that makes sense:
    - multishot-measure of 12 qubits x 10^4 trials: one marginal reduction +
      host replay, against the reference's per-trial reload (device copy) and
      sequential measure (app/src/api/multishot-measure.lisp:93-109), timed
      on 100 trials and scaled;
    - expectation of 8 two-Pauli operators (device copy + program + inner);
    - wavefunction wire bytes (big-endian, 16 B per amplitude) to the host;
    - a 4-operator depolarizing Kraus step on one qubit (two passes) against
      the reference's algorithm (copy, apply K_j, norm, until the sum reaches
      the draw; src/apply-gate.lisp:16-39), both on the device;
    - a 10-qubit density matrix (a 20-qubit vector) through a depolarized
      random circuit."""
    import random as pyrandom

    from qvm_gb300 import CudaPureState, Program, api, circuits
    from qvm_gb300.density import DensityQVM
    from qvm_gb300.noisy import make_pauli_noise_map

    out = {"qubits": n, "precision": "fp64"}
    gs = circuits.random_su_circuit(n, depth=6, seed=seed)
    prep = Program()
    prep.add_gates(gs)
    prep.plan(n, "fp64", fused=True, fusion_width=2)
    s = CudaPureState(n, "fp64")
    prep.run(s, fused=True)
    s.sync()

    def timed(fn, reps=3):
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            r = fn()
            best = min(best, time.perf_counter() - t0)
        return best, r

    # multishot-measure: 12 qubits, 10^4 trials
    qubits = list(range(0, n, 2))[:12]
    rng = pyrandom.Random(seed)
    t_ours, bits = timed(lambda: api.measure_trials(s, qubits, 10000, rng))
    work = CudaPureState(n, "fp64")

    def per_trial(trials):
        r = pyrandom.Random(seed)
        for _ in range(trials):
            work.copy_from(s)
            for q in qubits:
                work.measure(q, r.random())
        work.sync()
    t_ref100, _ = timed(lambda: per_trial(100), reps=1)
    out["multishot_measure"] = {"measured_qubits": len(qubits), "trials": 10000,
                                "ms": 1e3 * t_ours, "trials_per_s": 10000 / t_ours,
                                "per_trial_reload_ms_est": 1e3 * t_ref100 * 100,
                                "speedup": t_ref100 * 100 / t_ours}
    # expectation of 8 operators
    ops = [f"Z {a}\nZ {a + 1}" for a in range(0, 16, 2)]
    prep_quil = "\n".join(f"RY({0.1 * (q + 1)}) {q}" for q in range(n)) + "\nCNOT 0 1\nCNOT 2 3"
    t_exp, vals = timed(lambda: api.perform_expectation(prep_quil, ops, n), reps=2)
    out["expectation"] = {"operators": len(ops), "ms": 1e3 * t_exp,
                          "ms_per_operator_incl_prep": 1e3 * t_exp / len(ops)}
    # wire bytes
    t_wire, raw = timed(lambda: s.wavefunction_octets(), reps=2)
    out["wavefunction_octets"] = {"bytes": len(raw), "ms": 1e3 * t_wire,
                                  "GB_per_s": len(raw) / t_wire / 1e9}
    del raw
    # Kraus step vs the reference algorithm on the device
    kraus = make_pauli_noise_map(0.05, 0.05, 0.05)
    q0 = [3]

    def ours():
        s.apply_kraus(kraus, q0, 0.99)   # a late draw: every p_j is needed
        s.sync()
    t_k, _ = timed(ours)
    trial = CudaPureState(n, "fp64")

    def reference_algorithm():
        summed = 0.0
        for k in kraus:
            trial.copy_from(s)
            trial.apply_matrix(k, q0)
            summed += trial.norm() ** 2
            if summed >= 0.99:
                break
        trial.normalize()
        trial.sync()
    t_r, _ = timed(reference_algorithm)
    hmat = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)
    t_gate, _ = timed(lambda: (s.apply_matrix(hmat, q0), s.sync()))
    out["kraus_step"] = {"operators": len(kraus), "ms": 1e3 * t_k,
                         "reference_algorithm_ms": 1e3 * t_r, "speedup": t_r / t_k,
                         "plain_gate_ms": 1e3 * t_gate}
    trial.free()
    work.free()
    s.free()
    prep.free()
    # noisy density matrix: 10 qubits (20-qubit vector), depolarizing 1q noise on every H
    nd = 10
    dq = DensityQVM(nd, fused=True, fusion_width=4)
    for q in range(nd):
        dq.set_noisy_gate("H", [q], [k @ hmat for k in make_pauli_noise_map(0.01, 0.01, 0.01)])
    prog = "\n".join(f"H {q}" for q in range(nd)) + "\n" + "\n".join(
        f"CNOT {q} {q + 1}\nRZ({0.3 * q}) {q + 1}" for q in range(nd - 1))
    dq.load_program(prog)
    dq.run()
    dq.state.sync()

    def dens():
        dq.reset_quantum_state()
        dq.run()
        dq.state.sync()
    t_d, _ = timed(dens)
    ngates = nd + 2 * (nd - 1)
    out["density_matrix"] = {"qubits": nd, "vector_qubits": 2 * nd, "gates": ngates,
                             "ms": 1e3 * t_d, "gates_per_s": ngates / t_d,
                             "trace": float(np.sum(dq.probabilities()))}
    dq.free()
    return out


def run_random32(fw: int, tile: int, engine: str, shots: int = 4096, seed: int = 3,
                 runs: int = 3, plain: bool = True):
    """The random circuit at 32 qubits (depth 20, 960 gates): fused FP32
    (32 GiB state) with the tuned engine and the other of the FMA and
    tensor-core engines; fused FP64 in double-float tiles and the plain FP64 kernels (64 GiB
    states each).  Fidelity and max amplitude error of the tuned FP32 state
    against plain FP64, and the shots both draw from the same 4096 uniforms."""
    from qvm_gb300 import CudaPureState, Program, circuits
    from qvm_gb300.autotune import apply_engine
    n = 32
    gates = circuits.random_su_circuit(n, depth=20, seed=seed)
    G = len(gates)
    s32 = CudaPureState(n, "fp32")
    out = {"workload": f"random SU(2)/SU(4) circuit, {n} qubits, depth 20, {G} gates"}
    # the tuned engine, and beside it the other of FMA (fusion width 2) and
    # tensor cores (fusion width 5)
    legs = [("fp32_" + engine, (fw, tile, engine))]
    legs.append(("fp32_fma", (2, 13, "fma")) if engine == "tc" else ("fp32_tc", (5, 13, "tc")))
    for label, (f, t, e) in legs:
        prog = Program()
        prog.add_gates(gates)
        apply_engine(prog, e)
        prog.plan(n, "fp32", fused=True, fusion_width=f, tile_qubits=t)
        best = float("inf")
        for _ in range(runs + 1):
            s32.set_to_zero_state()
            ms, _ = prog.run_profiled(s32, fused=True)
            best = min(best, float(ms.sum()))
        out[label] = {"ms": best, "gates_per_s": G / (best / 1e3), "fusion_width": f,
                      "tile_qubits": t}
        prog.free()
    sdf = CudaPureState(n, "fp64")
    prog = Program()
    prog.add_gates(gates)
    prog.plan(n, "fp64", fused=True, fusion_width=2, tile_qubits=12)
    t0 = time.perf_counter()
    prog.run(sdf, fused=True)
    sdf.sync()
    out["fused_df64"] = {"ms": 1e3 * (time.perf_counter() - t0)}
    out["fused_df64"]["gates_per_s"] = G / (out["fused_df64"]["ms"] / 1e3)
    ref, ref_name = sdf, "fused FP64 (double-float tiles)"
    if plain:
        sp = CudaPureState(n, "fp64")
        t0 = time.perf_counter()
        prog.run(sp, fused=False)
        sp.sync()
        ms_p = 1e3 * (time.perf_counter() - t0)
        fdf, edf = sp.fidelity(sdf)
        out["plain_fp64"] = {"ms": ms_p, "gates_per_s": G / (ms_p / 1e3)}
        out["fused_df64"].update({"fidelity_vs_plain_fp64": fdf, "max_abs_err": edf})
        sdf.free()
        ref, ref_name = sp, "plain FP64 kernels"
    prog.free()
    # the state of the tuned FP32 engine against the FP64 reference state
    prog = Program()
    prog.add_gates(gates)
    apply_engine(prog, engine)
    prog.plan(n, "fp32", fused=True, fusion_width=fw, tile_qubits=tile)
    s32.set_to_zero_state()
    prog.run(s32, fused=True)
    f, err = ref.fidelity(s32)
    draws = np.random.default_rng(seed + 1).random(shots)
    same = int((ref.sample(draws) == s32.sample(draws)).sum())
    out["fidelity"] = {"fused_fp32_vs": ref_name, "fidelity": f, "one_minus": 1.0 - f,
                       "max_abs_err": err, "shots": shots, "identical_shots": same}
    prog.free()
    ref.free()
    s32.free()
    return out


def _serve_stream(work, drain_s: float):
    """Submit (offset, Request) pairs at their arrival times to a fresh server
    (HBM budget 180 GB, 16 workers); returns (t0, [(arrival, done, latency,
    n)]) for the requests that completed before the drain deadline."""
    from qvm_gb300.serve import Server
    srv = Server(hbm_budget=180e9, workers=16)
    subs = []
    t0 = time.perf_counter()
    for off, req in work:
        now = time.perf_counter() - t0
        if off > now:
            time.sleep(off - now)
        req.arrival = time.perf_counter()
        subs.append((req, srv.submit(req)))
    deadline = time.perf_counter() + drain_s
    done = []
    for req, f in subs:
        try:
            r = f.result(timeout=max(0.0, deadline - time.perf_counter()))
            done.append((req.arrival - t0, req.arrival - t0 + r.latency_s, r.latency_s, req.n))
        except Exception:
            pass
    srv.close_now()
    return t0, done


def _pct(xs, q):
    return float(np.percentile(np.asarray(xs) * 1e3, q)) if len(xs) else None


def run_serving(arrive_s: float = 1.5, drain_s: float = 60.0, seed: int = 5,
                steady_s: float = 12.0, load: float = 0.75):
    """Serving stream: Poisson arrivals of random-layer, QFT and QAOA programs
    with 10..30 qubits, depth 5..40, shots 1..1e4, FP32 or FP64, admitted by
    HBM bytes within 180 GB.
    - `offered`: the workload's own rate, 200 requests/s, for `arrive_s`
      seconds, then the queue drains.  Its completion rate is the engine's
      capacity on this mix (the device is saturated), and its latencies
      measure the backlog of the burst.
    - `steady`: arrivals at `load` x that capacity for `steady_s` seconds;
      jobs/s and p50/p99 latency over the requests that arrived between 2 s
      and steady_s - 2 s (start-up and drain excluded), a load the engine
      sustains."""
    from qvm_gb300.serve import serving_workload
    work = serving_workload(arrive_s, rate=200.0, seed=seed)
    _, done = _serve_stream(work, drain_s)
    span = max(d[1] for d in done) if done else float("nan")
    cap = len(done) / span if done else 0.0
    lat = [d[2] for d in done]
    offered = {"requests": len(work), "completed": len(done), "arrival_rate": 200.0,
               "arrivals_s": arrive_s, "window_s": span, "jobs_per_s": cap,
               "offered_over_capacity": 200.0 / cap if cap else None,
               "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
               "p50_ms_n_le_24": _pct([d[2] for d in done if d[3] <= 24], 50)}
    rate = load * cap
    work2 = serving_workload(steady_s, rate=rate, seed=seed + 1)
    _, done2 = _serve_stream(work2, drain_s)
    lo, hi = 2.0, steady_s - 2.0
    win = [d for d in done2 if lo <= d[0] <= hi]
    steady = {"arrival_rate": rate, "load_of_capacity": load, "arrivals_s": steady_s,
              "requests": len(work2), "completed": len(done2),
              "window": f"requests arriving in [{lo:.0f} s, {hi:.0f} s]",
              "window_requests": len(win),
              "jobs_per_s": len([d for d in done2 if lo <= d[1] <= hi]) / (hi - lo),
              "p50_ms": _pct([d[2] for d in win], 50), "p99_ms": _pct([d[2] for d in win], 99),
              "p50_ms_n_le_24": _pct([d[2] for d in win if d[3] <= 24], 50)}
    return {"qubits": "10..30", "budget_gb": 180, "offered": offered, "steady": steady}


def run_reference(args):
    """The reference arm: the oracle port of the reference's CPU algorithm
    (no SBCL here), all host cores, FP64.  One step = one fixed sample of the
    circuit (reference_sample: a third of a layer, 15 gates at 30 qubits,
    the layer's gate mix), applied in turn to one state; ms_per_step is the
    measured time of those steps."""
    ws, rank, _ = dist()
    if rank != 0:
        return
    from oracle import oracle as O
    from qvm_gb300 import circuits
    n = args.n
    gates = circuits.random_su_circuit(n, args.depth, args.seed)
    threads = os.cpu_count() or 1
    O.set_workers(threads, threshold=19)
    wf = O.zero_state(n)
    step_ms, done = [], 0
    for j in range(args.warmup + args.steps):
        sample = reference_sample(gates, n, j)
        t0 = time.perf_counter()
        for m, qs in sample:
            O.apply_matrix_operator(wf, m, qs)
        dt = time.perf_counter() - t0
        if j >= args.warmup:
            step_ms.append(1e3 * dt)
            done += len(sample)
    total_ms = float(np.sum(step_ms))
    value = done / (total_ms / 1e3)
    per = done // args.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Haar SU(2)/SU(4) circuit)", "impl": "reference",
            "config": {"workload": f"random SU(2)/SU(4) circuit, {n} qubits, depth "
                                   f"{args.depth}; one step = {per} of its gates (a third "
                                   f"of a layer: {n // 3} SU(2) + {n // 6} SU(4)), FP64, "
                                   f"applied in circuit order to one state",
                       "cpu": "oracle restatement of the reference's apply-matrix-operator "
                              "(no SBCL on this host)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} timed steps of {per} gates, "
                                       f"{total_ms / 1e3:.1f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _case_state(n, prec, seed=7):
    from qvm_gb300 import CudaPureState, Program, circuits
    s = CudaPureState(n, prec)
    p = Program()
    p.add_gates(circuits.random_su_circuit(n, depth=2, seed=seed))
    p.plan(n, prec, fused=True, fusion_width=2)
    p.run(s, fused=True)
    p.free()
    s.sync()
    return s


def case_sampler():
    """26-qubit FP64 state, 4096 shots: k_block_sums, k_scan_inclusive, k_sample."""
    s = _case_state(26, "fp64")
    draws = np.random.default_rng(1).random(4096)
    for _ in range(2):
        s.sample(draws, rule="cdf")
    s.free()
    return "sampled 2 x 4096 shots from a 26-qubit FP64 state"


def case_collapse():
    """26-qubit FP64 state: P(q=1) then force-measurement: k_prob_sum_*, k_collapse."""
    s = _case_state(26, "fp64")
    for q in (3, 20):
        p1 = s.excited_probability(q)
        s.force_measurement(1, q, p1)
    s.sync()
    s.free()
    return "two force-measurements on a 26-qubit FP64 state"


def case_perm():
    """SWAP q1,q20 as a plain pass: 27-qubit FP32 and 26-qubit FP64 (1 GiB each): k_perm."""
    from qvm_gb300 import CudaPureState, gates as G
    for n, prec in ((27, "fp32"), (26, "fp64")):
        s = CudaPureState(n, prec)
        for _ in range(2):
            s.apply_matrix(G.gate_matrix("SWAP"), [20, 1])
        s.sync()
        s.free()
    return "SWAP q1,q20 twice on 27-qubit FP32 and 26-qubit FP64 states"


def case_dense64():
    """A Haar SU(4) on q3,q17 of a 26-qubit FP64 state: k_dense<double, 2>."""
    from qvm_gb300 import CudaPureState, circuits
    s = CudaPureState(26, "fp64")
    rng = np.random.default_rng(2)
    for _ in range(2):
        s.apply_matrix(circuits.haar_special_unitary(rng, 4), [17, 3])
    s.sync()
    s.free()
    return "two SU(4) on a 26-qubit FP64 state"


def case_qaoa():
    """152 QAOA instances of 20 qubits (p = 4, 1024 shots; one per SM of
    the launch's grid, 1.2 GB of states): k_qaoa_batch."""
    from qvm_gb300.batch import QaoaBatch, random_qaoa_batch
    graphs, gam, bet = random_qaoa_batch(19, [20], 8, p=4, seed=4)
    b = QaoaBatch(graphs, gam, bet)
    draws = np.random.default_rng(4).random((len(graphs), 1024))
    for _ in range(2):
        b.run(draws)
    b.free()
    return f"2 runs of a {len(graphs)}-instance QAOA batch"


PROFILE_CASES = {"sampler": case_sampler, "collapse": case_collapse, "perm": case_perm,
                 "dense64": case_dense64, "qaoa": case_qaoa}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.case:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"case": args.case, "did": PROFILE_CASES[args.case]()}), flush=True)
        return
    ws, rank, local = dist()
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from qvm_gb300 import CudaPureState, Program, circuits
    from qvm_gb300.state import PRECISIONS  # noqa: F401

    n = args.n
    gates = circuits.random_su_circuit(n, args.depth, args.seed)
    G = len(gates)
    prog = Program()
    prog.add_gates(gates)
    s32 = CudaPureState(n, "fp32")
    stream = torch.cuda.ExternalStream(s32.stream())
    tuned = None
    from qvm_gb300.autotune import DEFAULT_CANDIDATES, apply_engine, autotune
    if args.fw == 0 or args.tile == 0 or args.engine == "auto":
        # untimed: pick fusion width, tile width and tile engine for this
        # circuit on this GPU
        cands = [(fw, t, e) for fw, t, e in DEFAULT_CANDIDATES["fp32"]
                 if args.fw in (0, fw) and args.tile in (0, t) and args.engine in ("auto", e)]
        (args.fw, args.tile, args.engine), table = autotune(prog, s32, "fp32", cands)
        tuned = {f"fw{fw}_t{t}_{e}": round(ms, 2) for (fw, t, e), ms in sorted(table.items())}
    apply_engine(prog, args.engine)
    stats = prog.plan(n, "fp32", fused=True, fusion_width=args.fw, tile_qubits=args.tile)

    def step():
        s32.set_to_zero_state()
        return prog.run_profiled(s32, fused=True)

    for _ in range(args.warmup):
        step()
    s32.sync()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    step_ms, tile_ms, launches = [], [], 0
    ev0.record(stream)
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ms, kinds = step()
        b.record(stream)
        b.synchronize()
        step_ms.append(a.elapsed_time(b))
        tile_ms.extend(ms[kinds == 3].tolist())
        launches += len(ms) + 1  # passes + the |0> amplitude kernel
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    total_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    total_ms = max_over_ranks(total_ms)
    value = whole_job_rate(G, args.steps, ws, total_ms)

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "data": "synthetic (seeded Haar SU(2)/SU(4) circuit)"}
    state_bytes = (1 << n) * 8
    result["config"] = {
        "workload": f"random SU(2)/SU(4) circuit, {n} qubits, depth {args.depth}, {G} gates, "
                    f"fused FP32 (fusion width {args.fw})",
        "passes": stats["passes"], "fused_blocks": stats["fused_blocks"],
        "fusion_width": args.fw, "tile_qubits": args.tile, "tile_engine": args.engine,
        "autotune_ms": tuned,
        "state_bytes": state_bytes,
        "l2": "state (%.1f GiB) is larger than L2; no flush needed" % (state_bytes / 2 ** 30),
        "parallelism": f"replicas x{ws}"}
    result["latency_ms"] = {"p50": float(np.percentile(step_ms, 50)),
                            "p99": float(np.percentile(step_ms, 99)), "what": "one circuit run"}
    peak, peak_kind = peaks()
    if tile_ms:
        avg = float(np.mean(tile_ms))
        ach = 2 * state_bytes / (avg / 1e3) / 1e9
        result["roofline"] = {"bound": "hbm", "kernel": "k_tile<float>", "achieved": ach,
                              "peak": peak, "unit": "GB/s", "frac": ach / peak,
                              "peak_source": peak_kind,
                              "algorithmic_bytes_per_launch": 2 * state_bytes,
                              "avg_launch_ms": avg,
                              "traffic": traffic_per_launch(n, args.engine),
                              "traffic_source": "ncu dram__bytes_read+write of one 26-qubit "
                                                "launch of the same engine, scaled by 2^(n-26)"}
    result["gpu_launches"] = launches
    result["clocks"] = clk

    # --- end to end through the public API with host buffers --------------------
    draws = np.random.default_rng(args.seed + 1).random(args.shots)
    e2e_ms = []
    h2d = d2h = 0
    for i in range(max(2, min(args.steps, 3))):
        t0 = time.perf_counter()
        p = Program()
        p.add_gates(gates)               # host gate matrices
        apply_engine(p, args.engine)
        st = p.plan(n, "fp32", fused=True, fusion_width=args.fw, tile_qubits=args.tile)
        s32.set_to_zero_state()
        p.run(s32, fused=True)           # plan upload + passes
        shots = s32.sample(draws)        # draws H2D, shot indices D2H
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        h2d = st.get("upload_bytes", 0) + draws.nbytes
        d2h = shots.nbytes
        p.free()
    result["e2e"] = {"value": G / (np.median(e2e_ms[1:]) / 1e3), "unit": UNIT,
                     "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                     "what": "Program build + plan + upload + run + 4096 shots via the C ABI"}

    # --- plain FP64 and fused double-float FP64, fidelity, shots --------------------
    if not args.no_fp64 and rank == 0:
        s64 = CudaPureState(n, "fp64")
        pp = Program()
        pp.add_gates(gates[:8])
        pp.run(s64, fused=False)       # warm-up on a prefix
        pp.free()
        s64.set_to_zero_state()
        s64.sync()
        st64 = torch.cuda.ExternalStream(s64.stream())
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st64)
        prog.run(s64, fused=False)
        b.record(st64)
        b.synchronize()
        ms64 = a.elapsed_time(b)
        # the same circuit in fused double-float tiles (FP64 state in HBM)
        pf = Program()
        pf.add_gates(gates)
        pf.plan(n, "fp64", fused=True, fusion_width=2, tile_qubits=12)
        sdf = CudaPureState(n, "fp64")
        pf.run(sdf, fused=True)        # untimed: plan upload
        dfbest = float("inf")
        for _ in range(2):
            sdf.set_to_zero_state()
            ms_df, _ = pf.run_profiled(sdf, fused=True)
            dfbest = min(dfbest, float(ms_df.sum()))
        fdf, errdf = s64.fidelity(sdf)
        sdf.free()
        pf.free()
        s32.set_to_zero_state()
        prog.run(s32, fused=True)
        f, err = s64.fidelity(s32)
        sh64 = s64.sample(draws)
        sh32 = s32.sample(draws)
        g64 = G / (ms64 / 1e3)
        result["plain_fp64"] = {"gates_per_s": g64, "ms": ms64,
                                "speedup_fused_fp32": value / ws / g64}
        result["fused_df64"] = {"gates_per_s": G / (dfbest / 1e3), "ms": dfbest,
                                "fidelity_vs_plain_fp64": fdf, "max_abs_err": errdf}
        result["fidelity"] = {"fused_fp32_vs_fp64": f, "one_minus": 1.0 - f,
                              "max_abs_err": err, "shots": int(args.shots),
                              "identical_shots": int((sh64 == sh32).sum())}
        s64.free()
    if not args.no_32q and rank == 0:
        s32.free()  # 8 GiB back before the 32-qubit states
        result["random32"] = run_random32(args.fw, args.tile, args.engine,
                                          plain=not args.no_32q_plain)
        s32 = CudaPureState(n, "fp32")
    if not args.no_qft and rank == 0:
        result[f"qft{args.qft_n}_fp64"] = run_qft_fp64(args.qft_n)
    if not args.no_plain_passes and rank == 0:
        result["plain_passes"] = run_plain_passes()
    if not args.no_layers and rank == 0:
        result["layers20_shots"] = run_layers_shots()
        result["engines_other"] = run_engines_other()
    if not args.no_endpoints and rank == 0:
        result["endpoints"] = run_endpoints()
    if not args.no_batch and rank == 0:
        result["batch_qaoa"] = run_qaoa_batch()
    if not args.no_serve and rank == 0:
        result["serving"] = run_serving()
    if not args.no_cpu and rank == 0 and ws == 1:
        cb = cpu_baseline(n, gates, args.cpu_steps, os.cpu_count() or 1)
        result["cpu_baseline"] = cb
        if "plain_fp64" in result:
            # precision-matched: FP64 on the GPU against the FP64 CPU port
            result["same_precision"] = {
                "cpu_fp64_gates_per_s": cb["value"],
                "plain_fp64_gates_per_s": result["plain_fp64"]["gates_per_s"],
                "fused_df64_gates_per_s": result["fused_df64"]["gates_per_s"],
                "plain_fp64_vs_cpu": result["plain_fp64"]["gates_per_s"] / cb["value"],
                "fused_df64_vs_cpu": result["fused_df64"]["gates_per_s"] / cb["value"],
                "fused_fp32_vs_cpu": value / ws / cb["value"]}
    if rank == 0:
        print(json.dumps(ordered(result)), flush=True)
    s32.free()
    if ws > 1:
        torch.distributed.destroy_process_group()


# Keys of the bench line, in print order: the contract's keys, then the
# detailed legs, then the summary figures last (a reader of only the end of
# the line still sees them).
_LEAD = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
         "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "gpu_launches",
         "config", "roofline", "clocks", "e2e", "cpu_baseline")
_TAIL = ("latency_ms", "random32", "qft28_fp64", "same_precision", "fused_df64", "plain_fp64",
         "fidelity")


def _round(x, digits=5):
    if isinstance(x, float):
        return float(f"{x:.{digits}g}") if np.isfinite(x) else x
    if isinstance(x, dict):
        return {k: _round(v, digits) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_round(v, digits) for v in x]
    return x


def ordered(result):
    out = {k: result[k] for k in _LEAD if k in result}
    middle = [k for k in result if k not in _LEAD and k not in _TAIL]
    for k in middle:
        out[k] = _round(result[k])
    for k in _TAIL:
        if k in result:
            # fidelities keep full precision; the other figures 5 digits
            out[k] = result[k] if k in ("fidelity", "fused_df64") else _round(result[k])
    return out


if __name__ == "__main__":
    main()
