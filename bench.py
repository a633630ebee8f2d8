#!/usr/bin/env python3
"""Benchmark: gate application on the 30-qubit complex128 random circuit (20
cycles of a Haar SU(2) on every qubit followed by CZ on 15 disjoint pairs),
the single-large-circuit configuration the GB300 target is quoted on.

A *step* applies the whole circuit (600 SU(2) + 300 CZ gates) to a state that
is resident in HBM, through StateVector.applyOperations as fused tile passes
computing in FP64 (the reference's arithmetic).  ``value`` counts the work
the circuit defines, independent of how it is executed: amplitude updates,
sum over gates of f * 2^n (f = fraction of amplitudes a gate changes: 1 for
SU(2), 1/4 for CZ), per second, in units of 1e9.  The CPU reference arm
counts the same units, so the two are directly comparable.  ``roofline``
gives the bytes the fused passes actually move (2 N S per pass) against the
measured HBM peak, ``fusion_gain`` the unfused-equivalent bytes, and
``e2e`` the same metric through the public binding with the state copied in
from pinned host memory and back out every step.  The 16 GiB state is far
larger than L2, so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path does not shard; replicas only) and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path[:0] = [str(REPO), str(REPO / "pennylane-lightning_gb300")]

METRIC = "30q c128 gate throughput (amplitude updates per second: sum over gates of f * 2^n, f = 1 for SU(2), 1/4 for CZ)"
UNIT = "G amplitude-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference", "cpu-sample", "cpu-configs"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--cycles", type=int, default=20)
    ap.add_argument("--tile-bits", type=int, default=None,
                    help="fixed fused tile size 2^t (0 = unfused); default: chosen during warm-up")
    ap.add_argument("--no-c64", action="store_true", help="skip the complex64 variant")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-circuits leg (config 2)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the autograd adjoint leg (config 3)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg (config 4)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the config-0 / config-3 GPU-and-host-cores comparison")
    ap.add_argument("--adjoint-qubits", type=int, default=28, help="config-3 register size (32: the 64 GiB variant)")
    ap.add_argument("--adjoint-layers", type=int, default=12, help="config-3 layers (6 for the 32-qubit variant)")
    ap.add_argument("--adjoint-fd", type=int, default=0,
                    help="also check this many sampled gradient entries by central finite differences")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="length of the config-4 arrival window replayed by the serving leg")
    return ap.parse_args()


def max_over_ranks(seconds: float, ws: int, device: str) -> float:
    """The slowest replica's time: every rank's timed region ends only when
    all replicas are done (no data-path collective; the path runs as
    independent replicas, one per GPU)."""
    if ws <= 1:
        return seconds
    import torch
    import torch.distributed as dist

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, ws: int, seconds: float) -> float:
    """Whole-job throughput: the units all replicas processed over the
    slowest replica's time (weak scaling)."""
    return ws * units_per_rank / seconds


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.idx)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- workload
def config1_circuit(n, cycles):
    from lightning_gb300.workloads import config1

    return config1(n, cycles, seed=1001)


def workload(n, cycles):
    from lightning_gb300.workloads import config1, unfused_bytes

    circuit, ham = config1(n, cycles, seed=1001)
    return circuit, ham, unfused_bytes


def rel_err(a, b):
    """(norm-relative difference, max relative difference over amplitudes
    with |b| >= 1e-2 max|b|) of two states."""
    nr = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    mag = np.abs(b)
    sel = mag >= 1e-2 * mag.max()
    return nr, float(np.max(np.abs(a[sel] - b[sel]) / mag[sel]))


def profile_value(kernel_tag: str, key: str):
    """A `key: value` line recorded in profiles/<tag>.md (ncu figures)."""
    p = REPO / "profiles" / f"{kernel_tag}.md"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.strip().startswith(key + ":"):
            try:
                return float(ln.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def traffic_from_profiles(kernel_tag: str):
    """Per-launch DRAM bytes (read + write) recorded in profiles/<tag>.md."""
    return profile_value(kernel_tag, "traffic_bytes_per_launch")


def gpu_arm(args) -> dict | None:
    import torch

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from lightning_gb300 import lightning_gb300_ops as ops

    peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text()) if (REPO / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    n, cycles = args.qubits, args.cycles
    circuit, ham, unfused_bytes = workload(n, cycles)
    alg_bytes = unfused_bytes(circuit, n, 16)  # unfused-equivalent bytes (gate by gate)
    updates = alg_bytes / 32.0  # amplitude updates: 2 f N S per gate with S = 16

    def ops_struct(cls):
        return cls([o.name for o in circuit], [o.params for o in circuit], [o.wires for o in circuit],
                    [False] * len(circuit), [o.matrix for o in circuit])

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    def timed_step(sv, S, stream, tb):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        passes = sv.applyOperations(S, tb)
        b.record(stream)
        sv.synchronize()
        return a.elapsed_time(b), passes

    S128 = ops_struct(ops.OpsStructC128)
    sv = ops.StateVectorC128(n)
    stream = torch.cuda.ExternalStream(sv.cuda_stream())
    # warm-up doubles as the tile-size choice among fused tiles of 2^t
    candidates = [10, 11, 12] if args.tile_bits is None else [args.tile_bits]
    tune = {}
    for w in range(max(args.warmup, 1)):
        tb = candidates[w % len(candidates)] if w < len(candidates) else best_tb
        ms, _ = timed_step(sv, S128, stream, tb)
        tune[tb] = min(ms, tune.get(tb, float("inf")))
        best_tb = min(tune, key=tune.get)
    for tb in candidates:
        if tb not in tune:
            tune[tb], _ = timed_step(sv, S128, stream, tb)
    best_tb = min(tune, key=tune.get)

    launches0 = ops.kernel_launches()
    step_ms, step_passes = [], []
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ms, passes = timed_step(sv, S128, stream, best_tb)
            step_ms.append(ms)
            step_passes.append(passes)
        barrier()
        wall = time.perf_counter() - t0
    launches = ops.kernel_launches() - launches0
    total_s = max_over_ranks(sum(step_ms) / 1e3, ws, "cuda")
    passes = step_passes[0]
    pass_bytes = 2.0 * (1 << n) * 16
    avg_launch_s = (total_s / args.steps) / passes
    achieved = pass_bytes / avg_launch_s / 1e9
    fp64_passes = bool(ops.set_c128_fp64_passes(True))  # the default; returns the setting in force
    if best_tb >= 9:
        kernel, tag = "k_tile_reg<double> (register-blocked fused tile pass, FP64)", "k_tile_reg_c128"
    else:
        kernel, tag = "k_tile_pass<double> (fused tile pass, FP64)", "k_tile_pass_c128"
    traffic = traffic_from_profiles(tag)
    if traffic is not None:  # recorded for a 30-qubit launch; traffic grows with the amplitudes
        traffic *= float(1 << n) / float(1 << 30)
    fp64_per_amp = profile_value(tag, "fp64_instructions_per_amplitude_per_pass")

    # unfused per-gate kernels on the first cycle (a cycle's gates are the
    # same mix in every cycle): the time of the whole circuit gate by gate
    per_cycle = len(circuit) // cycles
    S_cycle = ops.OpsStructC128([o.name for o in circuit[:per_cycle]], [o.params for o in circuit[:per_cycle]],
                                [o.wires for o in circuit[:per_cycle]], [False] * per_cycle,
                                [o.matrix for o in circuit[:per_cycle]])
    timed_step(sv, S_cycle, stream, 0)
    unfused_ms = timed_step(sv, S_cycle, stream, 0)[0] * cycles

    # expectation value of the 64-term Hamiltonian
    H = ops.observables.HamiltonianC128(
        ham.coeffs, [ops.observables.TensorProdObsC128(
            [ops.observables.NamedObsC128({"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}[c], [w])
             for c, w in zip(word, wires)]) for word, wires in zip(ham.words, ham.wires)])
    m = ops.MeasurementsC128(sv)
    m.expval(H)
    t = time.perf_counter()
    ev_val = m.expval(H)
    expval_ms = (time.perf_counter() - t) * 1e3

    # opt-in double-float passes: time, and accuracy against the FP64
    # passes on the same circuit at 26 qubits
    ops.set_c128_fp64_passes(False)
    try:
        timed_step(sv, S128, stream, best_tb)
        df_ms = min(timed_step(sv, S128, stream, best_tb)[0] for _ in range(2))
        n_acc = min(n, 26)
        circ_acc, _ = config1_circuit(n_acc, cycles)
        S_acc = ops.OpsStructC128([o.name for o in circ_acc], [o.params for o in circ_acc],
                                  [o.wires for o in circ_acc], [False] * len(circ_acc),
                                  [o.matrix for o in circ_acc])
        states = {}
        for fp64 in (False, True):
            ops.set_c128_fp64_passes(fp64)
            a_sv = ops.StateVectorC128(n_acc)
            a_sv.applyOperations(S_acc, best_tb)
            states[fp64] = a_sv.state()
            del a_sv
        df_nr, df_pr = rel_err(states[False], states[True])
        del states
    finally:
        ops.set_c128_fp64_passes(fp64_passes)

    # e2e through the binding: pinned host state in, circuit, state out
    host_in = torch.empty(1 << n, dtype=torch.complex128, pin_memory=True)
    host_out = torch.empty(1 << n, dtype=torch.complex128, pin_memory=True)
    host_in.zero_()
    host_in[0] = 1.0
    hin, hout = host_in.numpy(), host_out.numpy()
    e2e_steps = max(1, min(args.steps, 2))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sv.updateData(hin)
        sv.applyOperations(S128, best_tb)
        sv.getState(hout)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = (1 << n) * 16 + sum(o.matrix.nbytes for o in circuit if o.matrix is not None)
    d2h = (1 << n) * 16
    # the same through one binding call per gate (lightning.qubit's device
    # call pattern; queued and fused by the binding's lazy fusion)
    def per_gate_step():
        sv.updateData(hin)
        for o in circuit:
            if o.matrix is not None:
                sv.applyMatrix(o.matrix, o.wires, False)
            else:
                getattr(sv, o.name)(o.wires, False, o.params)
        sv.getState(hout)

    per_gate_step()  # warm-up
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        per_gate_step()
    barrier()
    pg_s = (time.perf_counter() - t0) / e2e_steps
    del sv

    step_s = total_s / args.steps
    fused_gbs = passes * pass_bytes / step_s / 1e9
    res = {
        "metric": METRIC, "value": replica_value(updates * args.steps, ws, total_s) / 1e9, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (f64 arithmetic)" if fp64_passes else "c128 (double-float arithmetic in fused passes)",
        "data": "synthetic (seeded Haar SU(2) + CZ circuit, seed 1001)",
        "config": {"workload": f"config1: {n} qubits complex128, {cycles} cycles x ({n} Haar SU(2) + {n // 2} CZ)",
                   "qubits": n, "gates_per_step": len(circuit), "amplitude_updates_per_step": updates,
                   "l2": (f"inputs larger than L2 ({(1 << n) * 16 / 2**30:g} GiB state)" if (1 << n) * 16 > 129e6
                          else f"state of {(1 << n) * 16 / 2**20:g} MiB fits L2"), "parallelism": f"replicas x{ws}",
                   "path": f"fused tile passes (FP64), 2^{best_tb} amplitudes per tile",
                   "tile_bits": best_tb, "passes_per_step": passes,
                   "tuning_ms_per_step": {str(k): round(v, 1) for k, v in sorted(tune.items())}},
        "e2e": {"value": updates / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "per_gate_calls": {"value": updates / pg_s / 1e9, "unit": UNIT, "ms_per_step": pg_s * 1e3,
                                   "path": f"{len(circuit)} binding calls per step (one per gate), lazy fusion"}},
        "roofline": {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": f"{peak_src} hbm_gbs", "traffic": traffic,
                     "algorithmic_bytes_per_launch": pass_bytes, "avg_launch_ms": avg_launch_s * 1e3,
                     "note": "fused-actual bytes (2 N S per pass) over the mean pass time.  A complex128 pass "
                             "computes in FP64, which GB300 executes at 1/64 of its FP32 rate (about 0.63 T "
                             "DFMA/s): the pass is bound by the FP64 pipe, not by HBM (fp64_pipe below)",
                     "fp64_pipe": {"fp64_instructions_per_amplitude_per_pass": fp64_per_amp,
                                   "source": f"profiles/{tag}.md (ncu)",
                                   "frac": profile_value(tag, "fp64_pipe_frac")},
                     "issue": {"metric": "smsp__issue_active (ncu, fraction of peak instruction issue)",
                               "frac": profile_value(tag, "issue_active_frac"),
                               "source": f"profiles/{tag}.md"}},
        "fusion_gain": {"unfused_equivalent_gbs": alg_bytes / step_s / 1e9, "fused_actual_gbs": fused_gbs,
                        "bytes_ratio": alg_bytes / (passes * pass_bytes), "unfused_ms_per_step": unfused_ms,
                        "time_ratio": unfused_ms / (step_s * 1e3),
                        "unfused_note": f"per-gate FP64 kernels on the first cycle x {cycles}"},
        "double_float": {"ms_per_step": df_ms, "value": updates / (df_ms / 1e3) / 1e9, "unit": UNIT,
                         "arithmetic": "double-float (hi + lo floats, ~48 significant bits, FP32 exponent range), "
                                       "opt-in (set_c128_fp64_passes(False))",
                         "accuracy_vs_fp64": {"qubits": n_acc, "norm_rel": df_nr, "per_amplitude_rel": df_pr,
                                              "per_amplitude_floor": "|a| >= 1e-2 max|a|"}},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "expval_64_terms": {"value": ev_val, "ms": expval_ms},
        "wall_s_timed": wall,
    }
    if not args.no_c64:
        S64 = ops_struct(ops.OpsStructC64)
        sv64 = ops.StateVectorC64(n)
        s64 = torch.cuda.ExternalStream(sv64.cuda_stream())
        t64 = {}
        # tile passes: complex64 registers of 22 qubits and more run
        # applyOperations as dense blocks while the tensor cores are on
        prev_tc = ops.set_tc_dense(False)
        try:
            for tb in ((11, 12) if args.tile_bits is None else (args.tile_bits,)):
                timed_step(sv64, S64, s64, tb)
                t64[tb] = timed_step(sv64, S64, s64, tb)[0]
        finally:
            ops.set_tc_dense(prev_tc)
        b64 = min(t64, key=t64.get)
        # dense-block fusion, fusion widths k = 2..6 (complex64 blocks of 4-6
        # wires on the tensor cores)
        def timed_blocks(svb, S, st, k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            nk = svb.applyOperationsBlocks(S, k)
            b.record(st)
            svb.synchronize()
            return a.elapsed_time(b), nk
        blk64 = {}
        for k in (2, 3, 4, 5, 6):
            timed_blocks(sv64, S64, s64, k)
            ms, nk = timed_blocks(sv64, S64, s64, k)
            blk64[k] = {"ms_per_step": ms, "kernels": nk, "value": updates / (ms / 1e3) / 1e9}
        kb = min(blk64, key=lambda k: blk64[k]["ms_per_step"])
        best = ("blocks", kb, blk64[kb]["ms_per_step"]) if blk64[kb]["ms_per_step"] < t64[b64] else \
            ("tiles", b64, t64[b64])
        res["c64"] = {"value": updates / (best[2] / 1e3) / 1e9, "unit": UNIT, "ms_per_step": best[2],
                      "path": (f"dense blocks of up to {kb} wires (tensor cores for 4-6 wires)" if best[0] == "blocks"
                               else f"fused tile passes, 2^{b64} amplitudes per tile"),
                      "tile_passes_ms_per_step": {str(k): round(v, 1) for k, v in sorted(t64.items())},
                      "fusion_width_sweep": {str(k): {"ms_per_step": round(v["ms_per_step"], 1),
                                                      "kernels": v["kernels"],
                                                      "value": v["value"]} for k, v in blk64.items()}}
        del sv64
        # the same sweep in complex128 (dense FP64 blocks on the CUDA cores)
        # at 26 qubits: a dense 2^k block costs 4 * 2^k FP64 multiply-adds per
        # amplitude, so this is a reference point, not a fast path
        n_sw = min(n, 26)
        circ_sw, _ = config1_circuit(n_sw, cycles)
        S_sw = ops.OpsStructC128([o.name for o in circ_sw], [o.params for o in circ_sw],
                                 [o.wires for o in circ_sw], [False] * len(circ_sw),
                                 [o.matrix for o in circ_sw])
        sv_sw = ops.StateVectorC128(n_sw)
        st_sw = torch.cuda.ExternalStream(sv_sw.cuda_stream())
        sweep128 = {}
        for k in (2, 3, 4, 5, 6):
            timed_blocks(sv_sw, S_sw, st_sw, k)
            ms, nk = timed_blocks(sv_sw, S_sw, st_sw, k)
            sweep128[str(k)] = {"ms_per_step": round(ms, 1), "kernels": nk}
        ms_t, p_t = timed_step(sv_sw, S_sw, st_sw, best_tb)
        res["c128_fusion_width_sweep"] = {"qubits": n_sw, "blocks": sweep128,
                                          "fused_tile_passes": {"ms_per_step": round(ms_t, 1), "passes": p_t}}
        del sv_sw
    if rank == 0:
        if not args.no_batch:
            res["batched"] = {"c128": batched_leg(ops, 128), "c64": batched_leg(ops, 64)}
        if not args.no_adjoint:
            res["adjoint"] = adjoint_leg(args.adjoint_qubits, args.adjoint_layers, args.adjoint_fd)
        if not args.no_serve:
            res["serving"] = serve_leg(args.serve_seconds)
    return res


# --------------------------------------------------------------------------- configs 2-4
def _plain_circuit(ops, packed, r, names, prec, lazy=False):
    """One circuit of a packed batch through the per-gate binding calls and
    per-observable expectation values (the plain per-call path: each gate
    applied at its call; lazy=True: the binding's lazy fusion)."""
    SV = ops.StateVectorC128 if prec == 128 else ops.StateVectorC64
    M = ops.MeasurementsC128 if prec == 128 else ops.MeasurementsC64
    s = "C128" if prec == 128 else "C64"
    NO, TP, HA = (getattr(ops.observables, k + s) for k in ("NamedObs", "TensorProdObs", "Hamiltonian"))
    n = int(packed.num_qubits[r])
    sv = SV(n)
    sv.set_lazy(lazy)
    for o in range(int(packed.op_offsets[r]), int(packed.op_offsets[r + 1])):
        name = names[int(packed.op_codes[o])]
        w = [int(x) for x in packed.op_wires[o] if x >= 0]
        getattr(sv, name)(w, False, [float(packed.op_params[o, 0])] if name != "CNOT" else [])
    m = M(sv)
    out = []
    for ob in range(int(packed.obs_offsets[r]), int(packed.obs_offsets[r + 1])):
        terms, coeffs = [], []
        for t in range(int(packed.term_offsets[ob]), int(packed.term_offsets[ob + 1])):
            fac = [NO(nm, [w]) for w in range(n) for nm, arr in (("PauliX", packed.term_x), ("PauliY", packed.term_y),
                                                                   ("PauliZ", packed.term_z)) if (int(arr[t]) >> w) & 1]
            terms.append(TP(fac))
            coeffs.append(float(packed.term_coeffs[t]))
        out.append(m.expval(HA(coeffs, terms)))
    return out


def batched_leg(ops, prec: int, plain_every: int = 32) -> dict:
    """Config 2: 4096 circuits through the batch engine (packed host arrays
    in, expectation values out: compilation, copies and device time all
    inside the timed region) vs the plain per-call path on every
    `plain_every`-th circuit."""
    from lightning_gb300.batch import BatchEngine, gate_codes
    from lightning_gb300.workloads import config2_packed

    packed = config2_packed(4096, seed=1002)
    names = {v: k for k, v in gate_codes().items()}
    eng = BatchEngine(prec)
    eng.run(packed)  # warm-up: tile-size autotuning, device arenas and pinned staging at full size
    t = time.perf_counter()
    vals = eng.run(packed)
    dt = time.perf_counter() - t
    st = eng.stats()
    df_leg = None
    if prec == 128:
        # the opt-in double-float passes on the same batch: throughput and the
        # largest deviation of its expectation values from the FP64 run's,
        # relative to each observable's sum |c| (the bound of |<O>|)
        prev = ops.set_c128_fp64_passes(False)
        try:
            eng_df = BatchEngine(prec)
            eng_df.run(packed)
            t = time.perf_counter()
            vals_df = eng_df.run(packed)
            dt_df = time.perf_counter() - t
        finally:
            ops.set_c128_fp64_passes(prev)
        to = np.asarray(packed.term_offsets, np.int64)
        norm = np.add.reduceat(np.abs(np.asarray(packed.term_coeffs, np.float64)), to[:-1])
        dev = np.abs(np.asarray(vals_df) - np.asarray(vals)) / norm
        df_leg = {"value": packed.num_circuits / dt_df, "unit": "circuits/s", "seconds": dt_df,
                  "arithmetic": "double-float passes (opt-in, set_c128_fp64_passes(False))",
                  "max_dev_vs_fp64_rel_sum_abs_c": float(dev.max()), "observables": int(dev.size)}
    lat = np.asarray(st["wave_done_ms"])[np.asarray(st["wave_of"], int)]
    sample = list(range(0, packed.num_circuits, plain_every))
    # warm-up of both per-call paths on the widest sampled circuit (first
    # launches of the fused kernels, pools)
    widest = max(sample, key=lambda r: int(packed.num_qubits[r]))
    _plain_circuit(ops, packed, widest, names, prec)
    _plain_circuit(ops, packed, widest, names, prec, lazy=True)
    plat = []
    t = time.perf_counter()
    for r in sample:
        t1 = time.perf_counter()
        _plain_circuit(ops, packed, r, names, prec)
        plat.append(time.perf_counter() - t1)
    pdt = time.perf_counter() - t
    plain = len(sample) / pdt
    t = time.perf_counter()
    for r in sample:
        _plain_circuit(ops, packed, r, names, prec, lazy=True)
    plain_lazy = len(sample) / (time.perf_counter() - t)
    extra = {}
    if df_leg is not None:
        df_leg["speedup_vs_plain"] = df_leg["value"] / plain
        extra["double_float"] = df_leg
    return {"metric": "config2 circuits/s", "value": packed.num_circuits / dt, "unit": "circuits/s",
            "circuits": packed.num_circuits, "seconds": dt, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "compile_ms": st["compile_ms"], "device_ms": st["device_ms"],
            "launches": st["launches"], "waves": st["waves"], "tile_bits": st["tile_bits"],
            "plain": {"value": plain, "unit": "circuits/s", "sample": f"every {plain_every}th circuit "
                      f"({len(sample)})", "p50_ms": float(np.percentile(plat, 50) * 1e3),
                      "p99_ms": float(np.percentile(plat, 99) * 1e3)},
            "plain_lazy_fusion": {"value": plain_lazy, "unit": "circuits/s",
                                  "note": "the same per-gate calls, queued and fused by the binding"},
            "speedup_vs_plain": packed.num_circuits / dt / plain,
            "speedup_vs_plain_lazy_fusion": packed.num_circuits / dt / plain_lazy, **extra}


def adjoint_leg(n: int = 28, layers: int = 12, fd: int = 0) -> dict:
    """Config 3: <H> of the 200-term Hamiltonian and its gradient in all
    rotation angles (1008 at 28 qubits x 12 layers, 576 at 32 x 6) through
    torch.autograd (checkpointed adjoint: two registers alive in the
    backward).  fd > 0: central finite differences (h = 1e-4) on that many
    sampled angles, as a check of the gradient at this size."""
    import torch

    from lightning_gb300.torch_adjoint import config3_circuit, expval

    circ, theta = config3_circuit(n=n, layers=layers)
    t = torch.tensor(theta, requires_grad=True)
    t0 = time.perf_counter()
    e = expval(t, circ)
    t1 = time.perf_counter()
    e.backward()
    t2 = time.perf_counter()
    out = {"metric": "config3 gradient s", "qubits": n, "layers": layers, "params": int(theta.size),
           "forward_s": t1 - t0, "backward_s": t2 - t1, "params_per_s": theta.size / (t2 - t0),
           "registers_in_backward": 2, "state_gib": (1 << n) * 16 / 2**30, "value": float(e.item())}
    if fd > 0:
        grad = t.grad.numpy()
        idx = np.random.default_rng(1003).choice(theta.size, size=min(fd, theta.size), replace=False)
        h, errs = 1e-4, []
        for j in idx:
            tp, tm = theta.copy(), theta.copy()
            tp[j] += h
            tm[j] -= h
            with torch.no_grad():
                d = (float(expval(torch.tensor(tp), circ)) - float(expval(torch.tensor(tm), circ))) / (2 * h)
            errs.append(abs(d - grad[j]))
        out["fd_check"] = {"params": [int(j) for j in idx], "h": h, "max_abs_err": float(max(errs))}
    return out


def serve_leg(seconds: float) -> dict:
    """Config 4: the Poisson request stream (2000 requests/s, n in 8..26,
    30 % adjoint) replayed for `seconds`, continuous batching, plus a serial
    per-request baseline on the first 200 requests."""
    from lightning_gb300 import lightning_gb300_ops as ops
    from lightning_gb300.batch import gate_codes
    from lightning_gb300.serve import Server
    from lightning_gb300.workloads import config4_packed

    packed, arrival, adjoint = config4_packed(duration=seconds)
    srv = Server(128)
    w = np.arange(min(64, packed.num_circuits))
    srv.run(packed.select(w), arrival[w] - arrival[0], adjoint[w])  # warm-up
    res = srv.run(packed, arrival, adjoint)
    out = {"metric": "config4 requests/s", **res.summary(), "window_s": seconds,
           "offered_per_s": packed.num_circuits / seconds}
    # the same stream with admission control: requests whose predicted wait
    # exceeds 1 s are refused at arrival
    slo = 1.0
    srv_adm = Server(128, slo_s=slo)
    srv_adm.run(packed.select(w), arrival[w] - arrival[0], adjoint[w])  # warm-up
    ra = srv_adm.run(packed, arrival, adjoint).summary()
    out["admission_control"] = {"slo_s": slo, "offered_per_s": packed.num_circuits / seconds,
                                "admitted": ra["requests"], "refused": ra["refused"],
                                "admitted_fraction": ra["requests"] / max(1, ra["offered"]),
                                "goodput_per_s": ra["throughput_per_s"], "p50_ms": ra["p50_ms"],
                                "p99_ms": ra["p99_ms"], "lanes": ra["lanes"]}
    # the same stream shape offered below capacity: latency without a backlog
    cap = out["throughput_per_s"]
    if cap > 0:
        rate = 0.7 * cap
        p2, a2, adj2 = config4_packed(rate=rate, duration=seconds, seed=1005)
        r2 = srv.run(p2, a2, adj2).summary()
        out["below_capacity"] = {"offered_per_s": p2.num_circuits / seconds, "requests": r2["requests"],
                                 "throughput_per_s": r2["throughput_per_s"], "p50_ms": r2["p50_ms"],
                                 "p99_ms": r2["p99_ms"], "rate": "0.7 x the measured throughput above"}
    names = {v: k for k, v in gate_codes().items()}
    srv.packed, srv.adjoint = packed, adjoint
    lat = []
    k = min(200, packed.num_circuits)
    t = time.perf_counter()
    for r in range(k):
        t1 = time.perf_counter()
        if adjoint[r]:
            srv.adjoint_one(r)
        else:
            _plain_circuit(ops, packed, r, names, 128)
        lat.append(time.perf_counter() - t1)
    out["serial"] = {"value": k / (time.perf_counter() - t), "unit": "requests/s", "sample": f"first {k} requests",
                     "service_p50_ms": float(np.percentile(lat, 50) * 1e3),
                     "service_p99_ms": float(np.percentile(lat, 99) * 1e3)}
    return out


# --------------------------------------------------------------------------- CPU legs
def cpu_setup():
    ncores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncores))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    from oracle.build_oracle import build_restatement
    from oracle.pyoracle import Oracle

    build_restatement()
    return Oracle("orc")


def cpu_sample_ops(n: int, cycles: int):
    """The CPU sample of the config-1 circuit: the first cycle's first 10
    SU(2) gates and first 5 CZ gates (the cycle's 2:1 mix of the two)."""
    circuit, _ = config1_circuit(n, cycles)
    first = circuit[: len(circuit) // cycles]
    su2 = [o for o in first if o.matrix is not None][:10]
    cz = [o for o in first if o.matrix is None][:5]
    return su2 + cz


def cpu_sample(orc, n_cpu: int, cycles: int, sv=None):
    """Time the CPU sample at n_cpu qubits on the host cores; returns
    (amplitude updates, seconds, gates, threads, state handle)."""
    from lightning_gb300.workloads import amplitude_updates

    ops_ = cpu_sample_ops(n_cpu, cycles)
    if sv is None:
        sv = orc.sv(n_cpu, np.complex128)
    t = time.perf_counter()
    for op in ops_:
        if op.matrix is not None:
            sv.apply_matrix(op.matrix, op.wires)
        else:
            sv.apply(op.name, op.wires)
    dt = time.perf_counter() - t
    return amplitude_updates(ops_, n_cpu), dt, len(ops_), orc.num_threads(), sv


def cpu_description(n_cpu: int, ng: int) -> str:
    return (f"{ng} gates of the config-1 circuit per step (the first cycle's first 10 Haar SU(2) and first 5 CZ) "
            f"at {n_cpu} qubits complex128; the LM-kernel restatement of lightning.qubit's algorithm with OpenMP on "
            f"the host cores (no AVX kernels on this host)")


def _median_time(f, reps=3):
    f()  # warm-up
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        f()
        ts.append(time.perf_counter() - t)
    return statistics.median(ts)


CONFIG3_CPU_QUBITS = 22  # config-3 size timed on both the host cores and the GPU


def cpu_configs_leg(orc) -> dict:
    """Configs 0 and 3 on the host cores (the oracle: the reference's
    algorithm with OpenMP): config 0 at its full size (20 qubits, 10 layers,
    600 parameters) and config 3 at 22 qubits (12 layers, 792 parameters,
    200-term Hamiltonian)."""
    from lightning_gb300.workloads import config0, config3, sum_z
    from oracle.pyoracle import pauli_sum_spec

    out = {"cores": orc.num_threads(), "host": host_cpu()}
    c0 = config0(20, 10, seed=1000)
    spec0 = pauli_sum_spec(sum_z(20).terms())
    sv = orc.sv(20, np.complex128)

    def fwd():
        sv.set_basis_state([0] * 20, list(range(20)))
        for op in c0:
            sv.apply(op.name, op.wires, False, op.params)
        sv.state()

    tp0 = list(range(sum(1 for o in c0 if o.params)))
    out["config0"] = {"qubits": 20, "params": len(tp0), "forward_s": _median_time(fwd),
                      "expval_s": _median_time(lambda: sv.expval_obs(spec0)),
                      "adjoint_s": _median_time(lambda: orc.sv(20, np.complex128).adjoint(
                          [o.as_dict() for o in c0], [spec0], tp0, apply_ops=True), reps=1)}
    n3 = CONFIG3_CPU_QUBITS
    c3, h3 = config3(n3, 12, seed=1003, nterms=200)
    tp3 = list(range(sum(1 for o in c3 if o.params)))
    out["config3"] = {"qubits": n3, "params": len(tp3), "terms": 200,
                      "adjoint_s": _median_time(lambda: orc.sv(n3, np.complex128).adjoint(
                          [o.as_dict() for o in c3], [pauli_sum_spec(h3.terms())], tp3, apply_ops=True), reps=1)}
    return out


def gpu_configs_leg(ops) -> dict:
    """Configs 0 and 3 on the GPU through the binding, as lightning.qubit's
    device calls it: one call per gate, then expval and the adjoint
    Jacobian (complex128)."""
    from lightning_gb300.workloads import config0, config3

    out = {}
    c0 = config0(20, 10, seed=1000)
    H = ops.observables.HamiltonianC128([1.0] * 20, [ops.observables.NamedObsC128("PauliZ", [q]) for q in range(20)])
    st = np.empty(1 << 20, np.complex128)
    holder = {}

    def fwd():
        sv = ops.StateVectorC128(20)
        for op in c0:
            getattr(sv, op.name)(op.wires, False, op.params)
        sv.getState(st)
        holder["sv"] = sv

    S0 = ops.OpsStructC128([o.name for o in c0], [o.params for o in c0], [o.wires for o in c0], [False] * len(c0),
                           [None] * len(c0))
    tp0 = list(range(sum(1 for o in c0 if o.params)))
    fwd_s = _median_time(fwd)
    m = ops.MeasurementsC128(holder["sv"])
    out["config0"] = {"qubits": 20, "params": len(tp0), "forward_s": fwd_s,
                      "expval_s": _median_time(lambda: m.expval(H)),
                      "adjoint_s": _median_time(lambda: ops.AdjointJacobianC128()(ops.StateVectorC128(20), [H], S0,
                                                                                    tp0, True))}
    n3 = CONFIG3_CPU_QUBITS
    c3, h3 = config3(n3, 12, seed=1003, nterms=200)
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    H3 = ops.observables.HamiltonianC128(list(h3.coeffs), [ops.observables.TensorProdObsC128(
        [ops.observables.NamedObsC128(names[c], [w]) for c, w in zip(wd, ws)]) for wd, ws in zip(h3.words, h3.wires)])
    S3 = ops.OpsStructC128([o.name for o in c3], [o.params for o in c3], [o.wires for o in c3], [False] * len(c3),
                           [None] * len(c3))
    tp3 = list(range(sum(1 for o in c3 if o.params)))
    out["config3"] = {"qubits": n3, "params": len(tp3), "terms": 200,
                      "adjoint_s": _median_time(lambda: ops.AdjointJacobianC128()(ops.StateVectorC128(n3), [H3], S3,
                                                                                    tp3, True))}
    return out


def reference_arm(args) -> None:
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    orc = cpu_setup()
    n_cpu = args.qubits
    sv = None
    for _ in range(args.warmup):
        *_, sv = cpu_sample(orc, n_cpu, args.cycles, sv)
    vals = []
    t_total = 0.0
    for _ in range(args.steps):
        u, t, ng, threads, sv = cpu_sample(orc, n_cpu, args.cycles, sv)
        vals.append(u / t / 1e9)
        t_total += t
    v = statistics.median(vals)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64 arithmetic)", "data": "synthetic",
        "config": {"workload": f"config1: {args.qubits} qubits complex128, {args.cycles} cycles x ({args.qubits} "
                               f"Haar SU(2) + {args.qubits // 2} CZ)", "qubits": args.qubits,
                   "sample": f"{ng} of the circuit's gates per step at {n_cpu} qubits (amplitude updates of the "
                             f"sampled gates over their time: the same metric)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": cpu_description(n_cpu, ng), "host": host_cpu()},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def host_cpu() -> str:
    """The host CPU model (lscpu) and core count, for the CPU numbers."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = {ln.split(":", 1)[0].strip(): ln.split(":", 1)[1].strip() for ln in out.splitlines() if ":" in ln}
        model = fields.get("Model name") or fields.get("Vendor ID", "")
    except (OSError, subprocess.TimeoutExpired):
        pass
    return f"{model or 'unknown'}, {os.cpu_count()} logical cores"


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    ws, rank, _ = dist_info()
    if args.impl == "cpu-configs":
        print(json.dumps(cpu_configs_leg(cpu_setup())))
        return
    if args.impl == "cpu-sample":
        # child process of the CPU baseline: OpenMP thread binding stays out
        # of the GPU process (its host threads compile circuits in parallel)
        orc = cpu_setup()
        n_cpu = args.qubits
        *_, sv = cpu_sample(orc, n_cpu, args.cycles)  # first touch of the host state
        u, t, ng, threads, _ = cpu_sample(orc, n_cpu, args.cycles, sv)
        print(json.dumps({"value": u / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                          "sample": cpu_description(n_cpu, ng) + f", {t:.1f} s", "host": host_cpu()}))
        return
    cpu = None
    if rank == 0 and not args.no_cpu:
        out = subprocess.run([sys.executable, str(Path(__file__).resolve()), "--impl", "cpu-sample", "--qubits",
                              str(args.qubits), "--cycles", str(args.cycles)], capture_output=True, text=True,
                             check=True)
        cpu = json.loads(out.stdout.strip().splitlines()[-1])
    cpu_cfg = None
    if rank == 0 and not args.no_cpu and not args.no_configs:
        out = subprocess.run([sys.executable, str(Path(__file__).resolve()), "--impl", "cpu-configs"],
                             capture_output=True, text=True, check=True)
        cpu_cfg = json.loads(out.stdout.strip().splitlines()[-1])
    res = gpu_arm(args)
    if rank == 0 and res is not None:
        res["cpu_baseline"] = cpu
        if not args.no_configs:
            from lightning_gb300 import lightning_gb300_ops as ops

            g = gpu_configs_leg(ops)
            cmp = {"gpu": g, "cpu": cpu_cfg}
            if cpu_cfg is not None:
                cmp["speedup"] = {c: {k: cpu_cfg[c][k] / g[c][k] for k in g[c] if k.endswith("_s")}
                                  for c in ("config0", "config3")}
            res["configs_0_3"] = cmp
        print(json.dumps(res))


if __name__ == "__main__":
    main()
