"""Continuous-batching request server on one GB300.

Requests (a circuit from |0..0>, a Pauli-sum Hamiltonian, optionally the
adjoint Jacobian of <H> with respect to every gate parameter) arrive over
time.  The server keeps a device-memory budget (2^n amplitudes per forward
request, three registers per adjoint request, 150 GB by default) and several
lanes, each a host thread with its own CUDA stream, that pull from their
queues independently, so work of different lanes overlaps on the device:

* two forward lanes (registers below / from `big_qubits`): every pass of the
  lane takes ALL queued requests the budget admits (requests that arrived
  while the previous batch was on the GPU join here) and runs them as one
  batch of the batch engine;
* `adjoint_lanes` adjoint lanes sharing one queue: a lane that finishes
  a request takes the next queued adjoint request the budget admits (up to
  `adjoint_take` at a time), so adjoint work is admitted per request while
  other requests are on the GPU; each lane runs on its own host thread,
  streams and buffer pool (fused forward pass, <H>, in-place adjoint
  sweep).

Admission control (`slo_s`): a request is refused at arrival when the
work queued ahead of it on its lane, at the lane's measured rate, would take
longer than `slo_s` (the lane's rate is learned from its completed batches:
cost units, gates x 2^n, x 4 for an adjoint, per second).  Under a load
beyond the device's capacity the admitted requests then keep a bounded
latency instead of all waiting on an ever longer queue; the refused ones
are reported.  Without `slo_s` every request is admitted.

Results of a request do not depend on what else is in flight: a forward
request's value is bit-identical to running it alone in a batch engine with
the same tile size, and an adjoint request runs exactly as it would alone.
"""
from __future__ import annotations

import collections
import ctypes as C
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import lightning_gb300_ops as ops
from ._capi import VP, call
from .batch import BatchEngine, PackedBatch, gate_codes


class MemoryBudget:
    def __init__(self, nbytes: int):
        self.free = int(nbytes)
        self.total = int(nbytes)
        self.cv = threading.Condition()

    def acquire(self, nbytes: int, block: bool = True) -> bool:
        with self.cv:
            if nbytes > self.total:
                raise ValueError(f"request needs {nbytes} bytes, more than the whole budget {self.total}")
            while self.free < nbytes:
                if not block:
                    return False
                self.cv.wait()
            self.free -= nbytes
            return True

    def release(self, nbytes: int):
        with self.cv:
            self.free += nbytes
            self.cv.notify_all()


class Admission:
    """Admission control by predicted wait.  Per lane kind: the cost queued
    or in flight, and the kind's completion rate (cost units per second over
    all its `parallel` lanes, an average of the completed batches weighted
    0.2 towards the newest).  A request is refused when the cost ahead of it
    plus its own, at that rate, exceeds `slo_s`; before a kind's first batch
    completes there is no rate yet and every request is admitted."""

    def __init__(self, slo_s: float | None, parallel):
        self.slo_s = None if slo_s is None else float(slo_s)
        self.parallel = [float(x) for x in parallel]
        self.backlog = [0.0] * len(self.parallel)
        self.rate = [None] * len(self.parallel)
        self.lock = threading.Lock()

    def offer(self, kind: int, cost: float) -> bool:
        with self.lock:
            r = self.rate[kind]
            if self.slo_s is not None and r is not None and (self.backlog[kind] + cost) / r > self.slo_s:
                return False
            self.backlog[kind] += cost
            return True

    def completed(self, kind: int, cost: float, seconds: float) -> None:
        with self.lock:
            self.backlog[kind] -= cost
            thr = cost / max(seconds, 1e-4) * self.parallel[kind]
            r = self.rate[kind]
            self.rate[kind] = thr if r is None else 0.8 * r + 0.2 * thr


@dataclass
class ServeResult:
    values: np.ndarray   # <H> per request
    jacobians: dict      # request -> d<H>/d(parameter of each rotation), adjoint requests
    arrival: np.ndarray  # seconds from the start
    start: np.ndarray    # seconds from the start when the request's batch began
    done: np.ndarray     # seconds from the start when its result was ready
    lane: np.ndarray     # lane index that served it
    batches: list = field(default_factory=list)  # (lane, size, seconds) per batch
    refused: np.ndarray = None  # requests refused by admission control

    @property
    def latency(self) -> np.ndarray:
        """Arrival to result, admitted requests only."""
        ok = self.admitted
        return self.done[ok] - self.arrival[ok]

    @property
    def admitted(self) -> np.ndarray:
        return ~self.refused if self.refused is not None else np.ones(self.done.size, bool)

    def summary(self) -> dict:
        lat = self.latency
        ok = self.admitted
        span = float(self.done[ok].max() - self.arrival.min()) if lat.size else 0.0
        busy = {}
        for li, size, sec in self.batches:
            k = "forward" if li < 2 else "adjoint"
            b = busy.setdefault(k, {"batches": 0, "requests": 0, "lane_seconds": 0.0})
            b["batches"] += 1
            b["requests"] += int(size)
            b["lane_seconds"] += float(sec)
        return {"requests": int(lat.size), "offered": int(self.done.size), "refused": int((~ok).sum()),
                "throughput_per_s": lat.size / span if span > 0 else 0.0,
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
                "mean_batch": float(np.mean([b[1] for b in self.batches])) if self.batches else 0.0,
                "batches": len(self.batches), "span_s": span, "lanes": busy}


class Server:
    def __init__(self, precision: int = 128, budget_bytes: float = 150e9, big_qubits: int = 20,
                 adjoint_lanes: int = 8, max_batch: int = 4096, tile_bits: int = 11, adjoint_share: float = 0.4,
                 adjoint_take: int = 1, slo_s: float | None = None):
        self.precision = int(precision)
        self.S = 16 if self.precision == 128 else 8
        # forward and adjoint lanes draw on separate shares of the budget, so
        # a backlog of one kind cannot starve the other
        self.budget = MemoryBudget(int(budget_bytes * (1.0 - adjoint_share)))
        self.adj_budget = MemoryBudget(int(budget_bytes * adjoint_share))
        self.big = int(big_qubits)
        self.max_batch = int(max_batch)
        self.tile_bits = int(tile_bits)
        self.adjoint_lanes = int(adjoint_lanes)
        self.adjoint_take = int(adjoint_take)
        self.slo_s = None if slo_s is None else float(slo_s)
        # forward lanes keep their engines (device arenas, tuned tile sizes)
        self.engines = [BatchEngine(self.precision, wave_bytes=int(budget_bytes)),
                        BatchEngine(self.precision, wave_bytes=int(budget_bytes))]
        # adjoint lanes: one engine each (its streams and buffer pool persist
        # across the requests the lane serves)
        self.adj_engines = [BatchEngine(self.precision, tile_bits=self.tile_bits,
                                        wave_bytes=int(budget_bytes * adjoint_share))
                            for _ in range(self.adjoint_lanes)]
        self._names = {v: k for k, v in gate_codes().items()}

    # ---------------------------------------------------------------- helpers
    def _bytes(self, r: int) -> int:
        n = max(int(self.packed.num_qubits[r]), 9)
        return (1 << n) * self.S * (3 if self.adjoint[r] else 1)

    def _costs(self) -> np.ndarray:
        """Cost units per request: gates x 2^n, x 4 for an adjoint request."""
        p = self.packed
        ngates = np.diff(np.asarray(p.op_offsets, np.int64)).astype(np.float64)
        c = ngates * np.exp2(np.asarray(p.num_qubits, np.float64))
        return c * np.where(self.adjoint, 4.0, 1.0)

    def _ops_struct(self, r: int):
        p = self.packed
        o0, o1 = int(p.op_offsets[r]), int(p.op_offsets[r + 1])
        names = [self._names[int(c)] for c in p.op_codes[o0:o1]]
        wires = [[int(x) for x in w if x >= 0] for w in p.op_wires[o0:o1]]
        params = [[float(v)] if nm in _ONE_PARAM else [] for nm, v in zip(names, p.op_params[o0:o1, 0])]
        OS = ops.OpsStructC128 if self.precision == 128 else ops.OpsStructC64
        return OS(names, params, wires, [bool(x) for x in p.op_inverse[o0:o1]], [None] * len(names))

    def _hamiltonian(self, r: int):
        p = self.packed
        s = "C128" if self.precision == 128 else "C64"
        NO = getattr(ops.observables, "NamedObs" + s)
        TP = getattr(ops.observables, "TensorProdObs" + s)
        HA = getattr(ops.observables, "Hamiltonian" + s)
        t0, t1 = int(p.term_offsets[r]), int(p.term_offsets[r + 1])
        n = int(p.num_qubits[r])
        terms = []
        for t in range(t0, t1):
            fac = []
            for w in range(n):
                for letter, arr in (("PauliX", p.term_x), ("PauliY", p.term_y), ("PauliZ", p.term_z)):
                    if (int(arr[t]) >> w) & 1:
                        fac.append(NO(letter, [w]))
            terms.append(TP(fac) if fac else NO("Identity", [0]))
        return HA([float(c) for c in p.term_coeffs[t0:t1]], terms)

    def adjoint_one(self, r: int, lane: int = 0):
        """<H> and its Jacobian for request r run alone (a batch of one on
        the lane's engine: the same computation as inside any batch)."""
        vals, jacs = self.adj_engines[lane].run_adjoint(self.packed.select([r]))
        return float(vals[0]), jacs[0][0]

    # ------------------------------------------------------------------- run
    def run(self, packed: PackedBatch, arrival: np.ndarray, adjoint: np.ndarray, speed: float = 1.0) -> ServeResult:
        """Replay the arrival schedule in real time (divided by `speed`) and
        serve every request; returns per-request results and timings."""
        self.packed, self.adjoint = packed, np.asarray(adjoint, bool)
        R = packed.num_circuits
        values = np.full(R, np.nan)
        jacs: dict = {}
        start = np.zeros(R)
        done = np.zeros(R)
        lane_of = np.zeros(R, np.int32)
        refused = np.zeros(R, bool)
        batches: list = []
        lock = threading.Lock()
        cost = self._costs()
        adm = Admission(self.slo_s, [1, 1, self.adjoint_lanes])

        def completed(li, got, seconds):
            adm.completed(li, float(cost[got].sum()), seconds)
        nl = 3  # two forward lanes; one queue shared by the adjoint lanes
        queues = [collections.deque() for _ in range(nl)]
        cvs = [threading.Condition() for _ in range(nl)]
        closing = threading.Event()
        errors: list = []
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def budget_of(li):
            return self.budget if li < 2 else self.adj_budget

        def take(li, limit):
            """Block for the first queued request of lane li, then take every
            queued request the lane's budget admits, up to `limit`."""
            bud = budget_of(li)
            with cvs[li]:
                while not queues[li]:
                    if closing.is_set():
                        return []
                    cvs[li].wait(0.05)
                first = queues[li][0]
            bud.acquire(self._bytes(first))
            got = [first]
            with cvs[li]:
                queues[li].popleft()
                while queues[li] and len(got) < limit:
                    r = queues[li][0]
                    if not bud.acquire(self._bytes(r), block=False):
                        break
                    got.append(queues[li].popleft())
            return got

        def forward_lane(li):
            eng = self.engines[li]
            try:
                while True:
                    got = take(li, self.max_batch)
                    if not got:
                        return
                    ts = now()
                    vals = eng.run(packed.select(got))
                    te = now()
                    fin = eng.done_ms()
                    for r in got:
                        self.budget.release(self._bytes(r))
                    completed(li, got, te - ts)
                    with lock:
                        for k, r in enumerate(got):
                            values[r] = vals[k]
                            start[r], lane_of[r] = ts, li
                            done[r] = min(te, ts + fin[k] / 1e3) if k < len(fin) else te
                        batches.append((li, len(got), te - ts))
            except Exception as e:  # surfaced after the run
                errors.append(e)
                closing.set()

        def adjoint_lane(li):
            eng = self.adj_engines[li - 2]
            try:
                while True:
                    got = take(2, self.adjoint_take)
                    if not got:
                        return
                    ts = now()
                    vals, js = eng.run_adjoint(packed.select(got))
                    te = now()
                    fin = eng.done_ms()
                    for r in got:
                        self.adj_budget.release(self._bytes(r))
                    completed(2, got, te - ts)
                    with lock:
                        for k, r in enumerate(got):
                            values[r], jacs[r] = vals[k], js[k][0]
                            start[r], lane_of[r] = ts, li
                            done[r] = min(te, ts + fin[k] / 1e3) if k < len(fin) else te
                        batches.append((li, len(got), te - ts))
            except Exception as e:
                errors.append(e)
                closing.set()

        threads = [threading.Thread(target=forward_lane, args=(0,), daemon=True),
                   threading.Thread(target=forward_lane, args=(1,), daemon=True)]
        threads += [threading.Thread(target=adjoint_lane, args=(2 + k,), daemon=True)
                    for k in range(self.adjoint_lanes)]
        for th in threads:
            th.start()
        for r in range(R):
            if errors:
                break
            wait = arrival[r] / speed - now()
            if wait > 0:
                time.sleep(wait)
            if self.adjoint[r]:
                li = 2
            else:
                li = 1 if packed.num_qubits[r] >= self.big else 0
            if not adm.offer(li, float(cost[r])):
                refused[r] = True
                with lock:
                    done[r] = now()
                continue
            with cvs[li]:
                queues[li].append(r)
                cvs[li].notify()
        # drain
        while not errors:
            with lock:
                finished = int(np.count_nonzero((done > 0) | refused))
            if finished == R:
                break
            time.sleep(0.01)
        closing.set()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return ServeResult(values, jacs, np.asarray(arrival, float) / speed, start, done, lane_of, batches, refused)


_ONE_PARAM = {"PhaseShift", "RX", "RY", "RZ", "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "ControlledPhaseShift",
              "CRX", "CRY", "CRZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus", "PSWAP",
              "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ", "GlobalPhase"}
