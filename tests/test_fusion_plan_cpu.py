"""Host-side checks of the fusion compiler (no GPU needed): the tile passes
plgb_ops_fusion_plan reports for a circuit.  The reference applies gates one
by one (LQ/StateVectorLQubit.hpp:378-391); fusion is this backend's own
scheduling, so these tests pin its plan properties rather than a reference
value: which passes run on the register kernel, how many passes a workload
needs, and which gates stay unfused."""
import numpy as np
import pytest

from lightning_gb300.workloads import config0, config1


def struct(ops_module, circuit, prec=128):
    OS = ops_module.OpsStructC128 if prec == 128 else ops_module.OpsStructC64
    return OS([o["name"] for o in circuit], [o.get("params", []) for o in circuit], [o["wires"] for o in circuit],
              [o.get("inverse", False) for o in circuit], [o.get("matrix") for o in circuit],
              [o.get("cwires", []) for o in circuit], [o.get("cvals", []) for o in circuit])


@pytest.mark.parametrize("prec", [64, 128])
@pytest.mark.parametrize("tile_bits", [11, 12])
def test_config1_30q_all_register_passes(ops_module, prec, tile_bits):
    # the headline workload: every pass is a register-kernel tile pass of the
    # requested size, and fusion keeps the pass count far below the 900 gates
    circuit, _ = config1(30, 20, seed=1001)
    plan = struct(ops_module, [op.as_dict() for op in circuit], prec).fusion_plan(30, tile_bits)
    assert all(p["tile"] and p["register_kernel"] and p["t"] == tile_bits for p in plan)
    # pass counts of the current scheduler (a regression shows as more passes)
    assert len(plan) <= {(128, 12): 24, (128, 11): 28, (64, 12): 25, (64, 11): 33}[(prec, tile_bits)]
    assert sum(p["ops"] for p in plan) < 900


def test_plan_is_deterministic(ops_module):
    circuit = [op.as_dict() for op in config0(16, 6, seed=5)]
    S = struct(ops_module, circuit)
    assert S.fusion_plan(16, 11) == S.fusion_plan(16, 11)


def test_multi_controlled_diagonals_are_fused(ops_module):
    # a phase with four or more controls is a diagonal on five or more bits;
    # without a cross-boundary form it claims its bits as tile-local bits
    rng = np.random.default_rng(11)
    n = 13
    circuit = []
    for _ in range(4):
        for q in range(n):
            circuit.append(dict(name="RY", wires=[q], params=[float(rng.uniform(0, 6))]))
        w = [int(x) for x in n - 9 + rng.choice(9, size=6, replace=False)]
        circuit.append(dict(name="PhaseShift", wires=w[:1], params=[0.4], cwires=w[1:], cvals=[True] * 5))
    plan = struct(ops_module, circuit).fusion_plan(n, 11)
    assert all(p["tile"] for p in plan), plan


def test_wide_dense_matrix_runs_unfused(ops_module):
    # a dense matrix on 3 wires has no tile-op form: it runs as its own
    # unfused segment between fused passes
    rng = np.random.default_rng(12)
    n = 12
    m = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    q, _ = np.linalg.qr(m)
    circuit = [dict(name="RX", wires=[k], params=[0.1 * k]) for k in range(n)]
    circuit.append(dict(name="QubitUnitary", wires=[0, 5, 9], matrix=q))
    circuit += [dict(name="RZ", wires=[k], params=[0.2 * k]) for k in range(n)]
    plan = struct(ops_module, circuit).fusion_plan(n, 10)
    unfused = [p for p in plan if not p["tile"]]
    assert len(unfused) == 1
    assert plan[0]["tile"] and plan[-1]["tile"]


def test_diagonals_merge_across_a_cnot_chain(ops_module):
    # the list schedule postpones diagonals until a gate needs them: in the
    # config-0 ansatz (RX RY RZ per qubit, then a CNOT ring) the diagonal
    # halves of a layer's rotations merge into about two groups per layer
    # and pass, where per-level placement staggered them along the chain
    # (the 22-qubit config-2 circuits went from 110 to 66 merged diagonals)
    n, layers = 14, 8
    circuit = [op.as_dict() for op in config0(n, layers, seed=7)]
    plan = struct(ops_module, circuit).fusion_plan(n, 11)
    rotations = sum(p["rotations"] for p in plan)
    diagonals = sum(p["diagonals"] for p in plan)
    assert rotations == n * layers  # RX RY RZ merge into one rotation per qubit and layer
    assert diagonals <= 2 * layers + 2 * len(plan), (diagonals, len(plan))


@pytest.mark.parametrize("n", [10, 11, 12])
def test_register_of_one_tile_runs_on_chip(ops_module, n):
    # a register no wider than its tile keeps every gate tile-local: each
    # pass is one register-kernel launch over the whole register, and the
    # pass count is set only by the 192 op records a pass stages
    from lightning_gb300.workloads import config2
    circuits = [c for c in config2(256, seed=1002) if c.n == n][:8]
    assert circuits
    for c in circuits:
        ops = [op.as_dict() for op in c.ops]
        plan = struct(ops_module, ops).fusion_plan(n, n)
        assert all(p["tile"] and p["register_kernel"] and p["t"] == n for p in plan)
        assert 1 <= len(plan) <= 3
        assert sum(p["ops"] for p in plan) <= 192 * len(plan)
