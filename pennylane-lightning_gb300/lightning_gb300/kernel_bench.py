"""Kernel micro-benchmarks: one hot kernel at a chosen register size, timed
with CUDA events on the state vector's own stream (median of `reps`).

    python -m lightning_gb300.kernel_bench tile128 26   # config-1 circuit, FP64 fused tile passes
    python -m lightning_gb300.kernel_bench dense6 26    # a 6-wire dense complex64 block (tensor cores)
    python -m lightning_gb300.kernel_bench blocks64 28  # config-1 circuit, complex64 dense blocks k = 2..6
    python -m lightning_gb300.kernel_bench expval 26    # 64-term Pauli Hamiltonian <H>, complex128

Each prints one line per case: time and the bytes a pass moves over that
time.  Used for the kernel profiles (the same command under ncu).
"""
from __future__ import annotations

import sys
import time

import numpy as np


def _timer(sv):
    import torch

    stream = torch.cuda.ExternalStream(sv.cuda_stream())

    def run(f, reps=5):
        f()
        sv.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            out = f()
            b.record(stream)
            sv.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts)), out

    return run


def _config1_ops(ops, n, prec):
    from .workloads import config1

    circ, ham = config1(n, 20, seed=1001)
    OS = ops.OpsStructC128 if prec == 128 else ops.OpsStructC64
    return OS([o.name for o in circ], [o.params for o in circ], [o.wires for o in circ], [False] * len(circ),
              [o.matrix for o in circ]), ham


def tile128(n: int) -> None:
    from . import lightning_gb300_ops as ops

    S, _ = _config1_ops(ops, n, 128)
    sv = ops.StateVectorC128(n)
    ms, passes = _timer(sv)(lambda: sv.applyOperations(S, 11), reps=2)
    print(f"{n}q c128 config-1 FP64 tile passes t=11: {ms:.1f} ms, {passes} passes, "
          f"{passes * 2 * (1 << n) * 16 / (ms / 1e3) / 1e9:.1f} GB/s fused-actual")


def dense6(n: int) -> None:
    from . import lightning_gb300_ops as ops

    rng = np.random.default_rng(1)
    q, _ = np.linalg.qr(rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64)))
    sv = ops.StateVectorC64(n)
    sv.set_lazy(False)
    run = _timer(sv)
    for wires, tag in (([n - 6 + i for i in range(6)], "six lowest bits"), (list(range(6)), "six highest bits"),
                       ([0, 3, n - 1, n - 4, 9, 14], "mixed bits")):
        # one dense block through the block-program path: its matrix image
        # is prepared once, so the timed call is the kernel and its error check
        S = ops.OpsStructC64(["QubitUnitary"], [[]], [wires], [False], [q.astype(np.complex64)])
        for tc in (True, False):
            ops.set_tc_dense(tc)
            ms, _ = run(lambda: sv.applyOperationsBlocks(S, 6))
            print(f"{n}q c64 dense 6-wire gate, {tag}, {'tensor cores' if tc else 'CUDA cores'}: {ms:.3f} ms, "
                  f"{2 * (1 << n) * 8 / (ms / 1e3) / 1e9:.1f} GB/s")
    ops.set_tc_dense(True)


def blocks64(n: int) -> None:
    from . import lightning_gb300_ops as ops

    S, _ = _config1_ops(ops, n, 64)
    sv = ops.StateVectorC64(n)
    run = _timer(sv)
    for tb in (11, 12):
        ms, p = run(lambda: sv.applyOperations(S, tb), reps=2)
        print(f"{n}q c64 config-1 tile passes t={tb}: {ms:.1f} ms ({p} passes)")
    for k in (2, 3, 4, 5, 6):
        ms, p = run(lambda: sv.applyOperationsBlocks(S, k), reps=2)
        print(f"{n}q c64 config-1 dense blocks k={k}: {ms:.1f} ms ({p} kernels)")


def expval(n: int) -> None:
    from . import lightning_gb300_ops as ops

    S, ham = _config1_ops(ops, n, 128)
    sv = ops.StateVectorC128(n)
    sv.applyOperations(S, 11)
    names = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    H = ops.observables.HamiltonianC128(list(ham.coeffs), [ops.observables.TensorProdObsC128(
        [ops.observables.NamedObsC128(names[c], [w]) for c, w in zip(wd, ws)]) for wd, ws in zip(ham.words, ham.wires)])
    m = ops.MeasurementsC128(sv)
    m.expval(H)
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        e = m.expval(H)
        ts.append(time.perf_counter() - t)
    print(f"{n}q c128 64-term <H> = {e!r}: {min(ts) * 1e3:.2f} ms")


CASES = {"tile128": tile128, "dense6": dense6, "blocks64": blocks64, "expval": expval}

if __name__ == "__main__":
    CASES[sys.argv[1]](int(sys.argv[2]) if len(sys.argv) > 2 else 26)
