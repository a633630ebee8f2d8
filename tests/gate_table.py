"""Gate names, wire counts and parameter counts of lightning.qubit.

Restates the tables in pennylane_lightning/core/gates/Constant.hpp
(gate_names, gate_wires, gate_num_params, controlled_gate_names,
generator_names) for use by the tests.  MultiRZ, GlobalPhase and PCPhase take
any number of wires (Constant.hpp multi_qubit_gates); they are listed with
wires=None.
"""

GATES = {
    # name: (num_wires, num_params)
    "Identity": (1, 0), "PauliX": (1, 0), "PauliY": (1, 0), "PauliZ": (1, 0),
    "Hadamard": (1, 0), "S": (1, 0), "SX": (1, 0), "T": (1, 0),
    "PhaseShift": (1, 1), "RX": (1, 1), "RY": (1, 1), "RZ": (1, 1), "Rot": (1, 3),
    "CNOT": (2, 0), "CY": (2, 0), "CZ": (2, 0), "SWAP": (2, 0),
    "IsingXX": (2, 1), "IsingXY": (2, 1), "IsingYY": (2, 1), "IsingZZ": (2, 1),
    "ControlledPhaseShift": (2, 1), "CRX": (2, 1), "CRY": (2, 1), "CRZ": (2, 1),
    "CRot": (2, 3), "SingleExcitation": (2, 1), "SingleExcitationMinus": (2, 1),
    "SingleExcitationPlus": (2, 1), "PSWAP": (2, 1),
    "Toffoli": (3, 0), "CSWAP": (3, 0),
    "DoubleExcitation": (4, 1), "DoubleExcitationMinus": (4, 1),
    "DoubleExcitationPlus": (4, 1),
    "MultiRZ": (None, 1), "GlobalPhase": (None, 1), "PCPhase": (None, 2),
}

CONTROLLED_GATES = [
    "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "PhaseShift",
    "RX", "RY", "RZ", "Rot", "SWAP", "IsingXX", "IsingXY", "IsingYY", "IsingZZ",
    "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
    "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus",
    "MultiRZ", "GlobalPhase", "PSWAP", "PCPhase",
]

GENERATORS = [
    "PhaseShift", "RX", "RY", "RZ", "IsingXX", "IsingXY", "IsingYY", "IsingZZ",
    "CRX", "CRY", "CRZ", "ControlledPhaseShift", "SingleExcitation",
    "SingleExcitationMinus", "SingleExcitationPlus", "DoubleExcitation",
    "DoubleExcitationMinus", "DoubleExcitationPlus", "PSWAP", "MultiRZ",
    "GlobalPhase",
]

CONTROLLED_GENERATORS = [
    "PhaseShift", "RX", "RY", "RZ", "IsingXX", "IsingXY", "IsingYY", "IsingZZ",
    "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
    "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus",
    "PSWAP", "MultiRZ", "GlobalPhase",
]


def gate_wires(name, rng, n, k_multi=3):
    """Random distinct wires for gate `name` on an n-qubit register."""
    nw = GATES[name][0]
    if nw is None:
        nw = k_multi
    return [int(w) for w in rng.choice(n, size=nw, replace=False)]


def gate_params(name, rng):
    npar = GATES[name][1]
    if name == "PCPhase":
        return [float(rng.uniform(0, 6.283185307179586)), 3.0]
    return [float(x) for x in rng.uniform(0, 6.283185307179586, size=npar)]
