"""Dense-block fusion on the host (no GPU): the blocks plgb_ops_block_plan
returns, multiplied out, equal the circuit's unitary (built column by column
by the oracle) for every block width, and no block exceeds its width."""
import numpy as np
import pytest

from helpers import seed_of


def circuit_unitary(oracle, n, ops):
    U = np.zeros((1 << n, 1 << n), np.complex128)
    for c in range(1 << n):
        o = oracle.sv(n, np.complex128)
        e = np.zeros(1 << n, np.complex128)
        e[c] = 1
        o.set_state(e)
        for op in ops:
            if op.get("matrix") is not None:
                o.apply_matrix(op["matrix"], op["wires"], op.get("inverse", False), op.get("cwires", ()),
                               op.get("cvals", ()))
            else:
                o.apply(op["name"], op["wires"], op.get("inverse", False), op.get("params", ()),
                        op.get("cwires", ()), op.get("cvals", ()))
        U[:, c] = o.state()
    return U


def block_unitary(n, blocks):
    U = np.eye(1 << n, dtype=np.complex128)
    idx = np.arange(1 << n)
    for b in blocks:
        t = b["targets"]  # first = most significant local bit (index bit positions)
        k = len(t)
        M = np.array([complex(re, im) for re, im in b["matrix"]]).reshape(1 << k, 1 << k)
        local = np.zeros(1 << n, np.int64)
        for m, bit in enumerate(t):
            local |= ((idx >> bit) & 1) << (k - 1 - m)
        rest = idx.copy()
        for bit in t:
            rest &= ~(1 << bit)
        G = np.zeros((1 << n, 1 << n), np.complex128)
        # G[i, j] = M[local(i), local(j)] when i and j agree outside the targets
        same = rest[:, None] == rest[None, :]
        G[same] = M[local[:, None], local[None, :]][same]
        U = G @ U
    return U


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_blocks_multiply_to_the_circuit(ops_module, oracle, k):
    from test_gpu_fusion import ops_struct, random_circuit

    n = 7
    rng = np.random.default_rng(seed_of("blocks", k))
    # gates that fit the width (wider ones would pass through unfused)
    ops = [o for o in random_circuit(rng, n, 60) if len(o["wires"]) + len(o.get("cwires", [])) <= k]
    S = ops_struct(ops_module, np.complex128, ops)
    plan = S.block_plan(n, k, matrices=True)
    assert all("matrix" in b and len(b["targets"]) <= k for b in plan)
    assert len(plan) < len(ops)
    U = circuit_unitary(oracle, n, ops)
    B = block_unitary(n, plan)
    assert np.max(np.abs(U - B)) < 1e-12


def test_config1_block_counts(ops_module):
    from lightning_gb300.workloads import config1

    circ, _ = config1(16, 4, seed=1001)
    S = ops_module.OpsStructC128([o.name for o in circ], [o.params for o in circ], [o.wires for o in circ],
                                 [False] * len(circ), [o.matrix for o in circ])
    counts = [len(S.block_plan(16, k)) for k in (1, 2, 3, 4, 5, 6)]
    assert counts[0] >= counts[-1] and all(c > 0 for c in counts)
    for k in (2, 4, 6):
        assert max(len(b["targets"]) for b in S.block_plan(16, k)) <= k
