"""Seeded synthetic circuits for the benchmark configurations.

No public benchmark suite is involved: every circuit, angle, matrix and
observable below is generated from ``numpy.random.default_rng(seed)`` with
seed = 1000 + configuration index, so a run is reproducible everywhere.

* config 0 — hardware-efficient ansatz: per layer RX, RY, RZ on every qubit,
  then a CNOT ring i -> i+1 mod n; observable sum_i Z_i.
* config 1 — 30-qubit random circuit: per cycle a Haar SU(2) on every qubit,
  then CZ on n/2 disjoint random pairs (each wire >= 24 is paired with a wire
  < 24, so every cycle exercises the small-stride bits); a 64-term Pauli
  Hamiltonian of weight 1..4 with N(0,1) coefficients.
* config 2 — batch of independent config-0 circuits with n ~ U{10..22} and
  depth ~ U{4..16}; each returns <sum Z_i> and 3 weight-2 Pauli strings.
* config 3 — strongly entangling ansatz: per layer Rot on each qubit (as
  RZ, RY, RZ for the adjoint) then CNOT(i, i + r mod n), r = (layer mod
  (n-1)) + 1; a 200-term Pauli Hamiltonian of weight <= 4.
* config 4 — open-loop Poisson request stream with n in 8..26,
  P(n) ~ 2^(-n/4), config-0 bodies of depth 2..12, 1..32-term Hamiltonians,
  30 % adjoint requests.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

TWO_PI = 2.0 * np.pi


@dataclass
class Op:
    name: str
    wires: list[int]
    params: list[float] = field(default_factory=list)
    matrix: np.ndarray | None = None
    inverse: bool = False

    def as_dict(self) -> dict:
        d = {"name": self.name, "wires": list(self.wires), "params": list(self.params), "inverse": self.inverse}
        if self.matrix is not None:
            d["matrix"] = self.matrix
        return d


@dataclass
class PauliSum:
    coeffs: list[float]
    words: list[str]
    wires: list[list[int]]

    def terms(self):
        return list(zip(self.coeffs, self.words, self.wires))


def haar_su2(rng) -> np.ndarray:
    """Haar-random SU(2): QR of a complex Ginibre 2x2 with the phase fix,
    then the determinant phase removed."""
    z = (rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    q = q * (d / np.abs(d))
    return q / np.sqrt(np.linalg.det(q))


def random_pauli_sum(rng, n: int, nterms: int, wmin: int = 1, wmax: int = 4) -> PauliSum:
    coeffs, words, wires = [], [], []
    for _ in range(nterms):
        w = int(rng.integers(wmin, wmax + 1))
        wires.append([int(x) for x in rng.choice(n, size=w, replace=False)])
        words.append("".join(rng.choice(list("XYZ"), size=w)))
        coeffs.append(float(rng.normal()))
    return PauliSum(coeffs, words, wires)


def sum_z(n: int) -> PauliSum:
    return PauliSum([1.0] * n, ["Z"] * n, [[q] for q in range(n)])


# --------------------------------------------------------------------- config 0
def config0(n: int = 20, layers: int = 10, seed: int = 1000) -> list[Op]:
    rng = np.random.default_rng(seed)
    angles = rng.uniform(0.0, TWO_PI, size=(layers, n, 3))
    ops: list[Op] = []
    for layer in range(layers):
        for q in range(n):
            ops.append(Op("RX", [q], [float(angles[layer, q, 0])]))
            ops.append(Op("RY", [q], [float(angles[layer, q, 1])]))
            ops.append(Op("RZ", [q], [float(angles[layer, q, 2])]))
        for q in range(n):
            ops.append(Op("CNOT", [q, (q + 1) % n]))
    return ops


# --------------------------------------------------------------------- config 1
def cz_pairs(rng, n: int, high_from: int) -> list[tuple[int, int]]:
    high = [q for q in range(n) if q >= high_from]
    low = [int(q) for q in rng.permutation([q for q in range(n) if q < high_from])]
    pairs = []
    for h in rng.permutation(high):
        pairs.append((low.pop(), int(h)))
    while len(low) >= 2:
        pairs.append((low.pop(), low.pop()))
    return pairs


def config1(n: int = 30, cycles: int = 20, seed: int = 1001, nterms: int = 64) -> tuple[list[Op], PauliSum]:
    rng = np.random.default_rng(seed)
    ops: list[Op] = []
    high_from = max(0, n - 6) if n >= 12 else n // 2
    for _ in range(cycles):
        for q in range(n):
            ops.append(Op("QubitUnitary", [q], matrix=haar_su2(rng)))
        for a, b in cz_pairs(rng, n, high_from):
            ops.append(Op("CZ", [a, b]))
    return ops, random_pauli_sum(rng, n, nterms)


def unfused_bytes(ops: list[Op], n: int, itemsize: int) -> float:
    """Algorithmic HBM bytes of applying `ops` one by one: 2 f N S per gate,
    f = fraction of amplitudes a gate changes (1 for dense / rotation gates,
    1/2 for CNOT/SWAP-like permutations, 1/4 for CZ-like phases)."""
    N = float(1 << n)
    frac = {"CZ": 0.25, "ControlledPhaseShift": 0.25, "CNOT": 0.5, "SWAP": 0.5, "PauliX": 1.0, "Toffoli": 0.25}
    return sum(2.0 * frac.get(op.name, 1.0) * N * itemsize for op in ops)


def amplitude_updates(ops: list[Op], n: int) -> float:
    """Work of applying `ops`, independent of how it is executed: sum over
    gates of f * 2^n amplitude updates (f as in unfused_bytes)."""
    return unfused_bytes(ops, n, 1) / 2.0


# --------------------------------------------------------------------- config 2
@dataclass
class BatchCircuit:
    n: int
    ops: list[Op]
    observables: list[PauliSum]


def config2(num: int = 4096, seed: int = 1002) -> list[BatchCircuit]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(num):
        n = int(rng.integers(10, 23))
        depth = int(rng.integers(4, 17))
        body = config0(n, depth, seed=int(rng.integers(0, 2**31 - 1)))
        obs = [sum_z(n)] + [random_pauli_sum(rng, n, 1, 2, 2) for _ in range(3)]
        out.append(BatchCircuit(n, body, obs))
    return out


def config2_packed(num: int = 4096, seed: int = 1002):
    """config2 in the batch engine's packed layout, built with array
    operations (same circuits and observables as config2)."""
    from .batch import MAX_WIRES_PER_OP, PackedBatch, code_of, pauli_masks

    rx, ry, rz, cnot = code_of("RX"), code_of("RY"), code_of("RZ"), code_of("CNOT")
    rng = np.random.default_rng(seed)
    nq, codes, wires, params = [], [], [], []
    op_off, term_off, coeffs, xs, ys, zs = [0], [0], [], [], [], []
    for _ in range(num):
        n = int(rng.integers(10, 23))
        depth = int(rng.integers(4, 17))
        angles = np.random.default_rng(int(rng.integers(0, 2**31 - 1))).uniform(0.0, TWO_PI, size=(depth, n, 3))
        obs = [sum_z(n)] + [random_pauli_sum(rng, n, 1, 2, 2) for _ in range(3)]
        per_layer = 4 * n
        c = np.empty((depth, per_layer), np.int32)
        c[:, :3 * n] = np.tile(np.array([rx, ry, rz], np.int32), n)
        c[:, 3 * n:] = cnot
        w = np.full((depth, per_layer, MAX_WIRES_PER_OP), -1, np.int32)
        q = np.arange(n, dtype=np.int32)
        w[:, :3 * n, 0] = np.repeat(q, 3)
        w[:, 3 * n:, 0] = q
        w[:, 3 * n:, 1] = (q + 1) % n
        pr = np.zeros((depth, per_layer, 3), np.float64)
        pr[:, :3 * n, 0] = angles.reshape(depth, 3 * n)
        nq.append(n)
        codes.append(c.reshape(-1))
        wires.append(w.reshape(-1, MAX_WIRES_PER_OP))
        params.append(pr.reshape(-1, 3))
        op_off.append(op_off[-1] + depth * per_layer)
        for o in obs:
            for cf, word, ws in zip(o.coeffs, o.words, o.wires):
                x, y, z = pauli_masks(word, ws)
                coeffs.append(cf)
                xs.append(x)
                ys.append(y)
                zs.append(z)
            term_off.append(len(coeffs))
    m = op_off[-1]
    return PackedBatch(np.asarray(nq, np.int32), np.asarray(op_off, np.int64), np.concatenate(codes),
                       np.concatenate(wires), np.concatenate(params), np.zeros(m, np.uint8),
                       np.arange(0, 4 * num + 1, 4, dtype=np.int64), np.asarray(term_off, np.int64),
                       np.asarray(coeffs, np.float64), np.asarray(xs, np.uint64), np.asarray(ys, np.uint64),
                       np.asarray(zs, np.uint64))


# --------------------------------------------------------------------- config 3
def config3(n: int = 28, layers: int = 12, seed: int = 1003, nterms: int = 200) -> tuple[list[Op], PauliSum]:
    rng = np.random.default_rng(seed)
    ops: list[Op] = []
    for layer in range(layers):
        r = (layer % (n - 1)) + 1
        ang = rng.uniform(0.0, TWO_PI, size=(n, 3))
        for q in range(n):
            phi, theta, omega = (float(x) for x in ang[q])
            # Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi), as the
            # adjoint transforms decompose it
            ops.append(Op("RZ", [q], [phi]))
            ops.append(Op("RY", [q], [theta]))
            ops.append(Op("RZ", [q], [omega]))
        for q in range(n):
            ops.append(Op("CNOT", [q, (q + r) % n]))
    return ops, random_pauli_sum(rng, n, nterms, 1, 4)


# --------------------------------------------------------------------- config 4
@dataclass
class Request:
    rid: int
    arrival: float
    n: int
    ops: list[Op]
    ham: PauliSum
    adjoint: bool


def config4_packed(rate: float = 2000.0, duration: float = 60.0, seed: int = 1004, n_max: int = 26):
    """The request stream in the batch engine's packed layout, generated
    with array operations.  Returns (packed, arrival seconds, adjoint flags):
    request r is circuit r of `packed` with one observable, its Hamiltonian.

    Per request: Poisson arrival at `rate`; n in 8..26 with P(n) ~ 2^(-n/4);
    a config-0 body of depth U{2..12}; a Hamiltonian of U{1..32} Pauli terms
    of weight U{1..min(4, n)} on distinct wires, letters U{X, Y, Z},
    coefficients N(0, 1); 30 % of the requests ask for the adjoint Jacobian."""
    from .batch import MAX_WIRES_PER_OP, PackedBatch, code_of

    rng = np.random.default_rng(seed)
    expect = int(rate * duration * 1.2) + 64
    gaps = rng.exponential(1.0 / rate, size=expect)
    arrival = np.cumsum(gaps)
    arrival = arrival[arrival < duration]
    R = arrival.size
    ns_all = np.arange(8, 27)
    pn = 2.0 ** (-ns_all / 4.0)
    pn /= pn.sum()
    ns = np.minimum(rng.choice(ns_all, size=R, p=pn), n_max).astype(np.int32)
    depth = rng.integers(2, 13, size=R)
    seeds = rng.integers(0, 2**31 - 1, size=R)
    nterms = rng.integers(1, 33, size=R)
    adjoint = rng.random(R) < 0.3

    rx, ry, rz, cnot = code_of("RX"), code_of("RY"), code_of("RZ"), code_of("CNOT")
    nops = (4 * ns * depth).astype(np.int64)
    op_off = np.concatenate([[0], np.cumsum(nops)]).astype(np.int64)
    M = int(op_off[-1])
    codes = np.empty(M, np.int32)
    wires = np.full((M, MAX_WIRES_PER_OP), -1, np.int32)
    params = np.zeros((M, 3), np.float64)
    # layout of a layer of an n-qubit body: 3n rotations (RX, RY, RZ per
    # wire) then n CNOTs; build one template per n and tile it
    tmpl = {}
    for n in range(8, 27):
        q = np.arange(n, dtype=np.int32)
        c = np.concatenate([np.tile(np.array([rx, ry, rz], np.int32), n), np.full(n, cnot, np.int32)])
        w = np.full((4 * n, MAX_WIRES_PER_OP), -1, np.int32)
        w[:3 * n, 0] = np.repeat(q, 3)
        w[3 * n:, 0] = q
        w[3 * n:, 1] = (q + 1) % n
        tmpl[n] = (c, w)
    term_off = np.concatenate([[0], np.cumsum(nterms)]).astype(np.int64)
    T = int(term_off[-1])
    coeffs = np.empty(T, np.float64)
    tx = np.zeros(T, np.uint64)
    ty = np.zeros(T, np.uint64)
    tz = np.zeros(T, np.uint64)
    for r in range(R):
        n, d = int(ns[r]), int(depth[r])
        c, w = tmpl[n]
        o0, o1 = int(op_off[r]), int(op_off[r + 1])
        codes[o0:o1] = np.tile(c, d)
        wires[o0:o1] = np.tile(w, (d, 1))
        sub = np.random.default_rng(int(seeds[r]))
        ang = sub.uniform(0.0, TWO_PI, size=(d, n, 3))
        p = params[o0:o1].reshape(d, 4 * n, 3)
        p[:, :3 * n, 0] = ang.reshape(d, 3 * n)
        k = int(nterms[r])
        wmax = min(4, n)
        wt = sub.integers(1, wmax + 1, size=k)
        perm = np.argsort(sub.random((k, n)), axis=1)[:, :wmax]
        letters = sub.integers(0, 3, size=(k, wmax))
        t0 = int(term_off[r])
        coeffs[t0:t0 + k] = sub.normal(size=k)
        bits = np.left_shift(np.uint64(1), perm.astype(np.uint64))
        live = np.arange(wmax)[None, :] < wt[:, None]
        for L, arr in ((0, tx), (1, ty), (2, tz)):
            sel = live & (letters == L)
            arr[t0:t0 + k] = np.bitwise_or.reduce(np.where(sel, bits, np.uint64(0)), axis=1)
    packed = PackedBatch(ns, op_off, codes, wires, params, np.zeros(M, np.uint8),
                         np.arange(R + 1, dtype=np.int64), term_off, coeffs, tx, ty, tz)
    return packed, arrival, adjoint


def config4(rate: float = 2000.0, duration: float = 60.0, seed: int = 1004, n_max: int = 26) -> list[Request]:
    """config4_packed as Request objects (for small streams)."""
    from .batch import gate_codes

    packed, arrival, adjoint = config4_packed(rate, duration, seed, n_max)
    names = {v: k for k, v in gate_codes().items()}
    reqs = []
    for r in range(packed.num_circuits):
        o0, o1 = int(packed.op_offsets[r]), int(packed.op_offsets[r + 1])
        ops = []
        for o in range(o0, o1):
            name = names[int(packed.op_codes[o])]
            ws = [int(x) for x in packed.op_wires[o] if x >= 0]
            ops.append(Op(name, ws, [float(packed.op_params[o, 0])] if name != "CNOT" else []))
        t0, t1 = int(packed.term_offsets[r]), int(packed.term_offsets[r + 1])
        coeffs, words, wires = [], [], []
        for t in range(t0, t1):
            word, ws = [], []
            for w in range(int(packed.num_qubits[r])):
                for letter, arr in (("X", packed.term_x), ("Y", packed.term_y), ("Z", packed.term_z)):
                    if (int(arr[t]) >> w) & 1:
                        word.append(letter)
                        ws.append(w)
            coeffs.append(float(packed.term_coeffs[t]))
            words.append("".join(word))
            wires.append(ws)
        reqs.append(Request(r, float(arrival[r]), int(packed.num_qubits[r]), ops, PauliSum(coeffs, words, wires),
                            bool(adjoint[r])))
    return reqs
