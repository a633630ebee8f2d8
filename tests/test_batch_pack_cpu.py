"""Packed batch layout (no GPU): the vectorised config-2 generator equals the
generic packer, sub-batch selection keeps every array consistent, and the
gate-code table is the library's."""
import numpy as np
import pytest

from lightning_gb300 import batch
from lightning_gb300.workloads import Op, PauliSum, config2, config2_packed


def test_config2_packed_equals_generic_pack():
    a = config2_packed(16, seed=1002)
    b = batch.pack(config2(16, seed=1002))
    for f in a.__dataclass_fields__:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_select_roundtrip():
    a = config2_packed(8, seed=3)
    s = a.select([5, 2])
    assert s.num_circuits == 2 and s.num_observables == 8
    for k, c in enumerate([5, 2]):
        o0, o1 = a.op_offsets[c], a.op_offsets[c + 1]
        p0, p1 = s.op_offsets[k], s.op_offsets[k + 1]
        assert np.array_equal(a.op_codes[o0:o1], s.op_codes[p0:p1])
        assert np.array_equal(a.op_params[o0:o1], s.op_params[p0:p1])
    full = a.select(range(8))
    for f in a.__dataclass_fields__:
        assert np.array_equal(getattr(a, f), getattr(full, f)), f


def test_gate_codes_and_masks():
    codes = batch.gate_codes()
    assert codes["PauliX"] != codes["CNOT"] and "DoubleExcitation" in codes and "QubitUnitary" not in codes
    assert batch.pauli_masks("XYZ", [0, 3, 5]) == (1, 8, 32)
    with pytest.raises(ValueError):
        batch.pauli_masks("Q", [0])
    with pytest.raises(ValueError):
        batch.pack([type("C", (), {"n": 2, "ops": [Op("Nope", [0])], "observables": []})()])
    p = batch.pack([type("C", (), {"n": 2, "ops": [Op("RX", [1], [0.5], inverse=True)],
                                   "observables": [PauliSum([2.0], ["ZX"], [[0, 1]])]})()])
    assert p.op_inverse.tolist() == [1] and p.op_wires.tolist() == [[1, -1, -1, -1]]
    assert p.term_z.tolist() == [1] and p.term_x.tolist() == [2] and p.term_coeffs.tolist() == [2.0]
