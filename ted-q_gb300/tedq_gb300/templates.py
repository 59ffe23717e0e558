"""Circuit templates.

``HardwareEfficient`` mirrors the reference's template
(tedq/templates/layers.py:65-115): per layer RY and RZ on every qubit, then
CNOTs on (i-1, i) for even i followed by odd i; a final RY, RZ layer unless
``final_layer=False``.  ``hea_spec`` returns the same circuit as a neutral
description (the dict format ``Circuit.from_spec`` records).
"""

import numpy as np

from . import operators as O


def _cnot_pairs(n):
    pairs = [(i - 1, i) for i in range(2, n, 2)]
    pairs += [(i - 1, i) for i in range(1, n, 2)]
    return pairs


class HardwareEfficient:
    def __init__(self, n_wires, depth, params, final_layer=True):
        params = np.asarray(params)
        for i in range(depth):
            for j in range(n_wires):
                O.RY(params[2 * i][j], qubits=[j])
                O.RZ(params[2 * i + 1][j], qubits=[j])
            for a, b in _cnot_pairs(n_wires):
                O.CNOT(qubits=[a, b])
        if final_layer:
            for j in range(n_wires):
                O.RY(params[2 * depth][j], qubits=[j])
                O.RZ(params[2 * depth + 1][j], qubits=[j])


def hea_spec(n_wires, depth, params=None, final_layer=False, measure="z_each"):
    """Neutral description of the hardware-efficient ansatz with <Z_i> outputs."""
    layers = depth + (1 if final_layer else 0)
    if params is None:
        params = np.zeros((2 * layers, n_wires))
    params = np.asarray(params, dtype=np.float64).reshape(2 * layers, n_wires)
    gates = []
    for i in range(depth):
        for j in range(n_wires):
            gates.append({"name": "RY", "qubits": [j], "params": [float(params[2 * i][j])], "trainable": [0]})
            gates.append({"name": "RZ", "qubits": [j], "params": [float(params[2 * i + 1][j])], "trainable": [0]})
        for a, b in _cnot_pairs(n_wires):
            gates.append({"name": "CNOT", "qubits": [a, b], "params": [], "trainable": []})
    if final_layer:
        for j in range(n_wires):
            gates.append({"name": "RY", "qubits": [j], "params": [float(params[2 * depth][j])], "trainable": [0]})
            gates.append({"name": "RZ", "qubits": [j], "params": [float(params[2 * depth + 1][j])], "trainable": [0]})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n_wires)]
    return {"n": n_wires, "gates": gates, "meas": meas, "init_state": None}
