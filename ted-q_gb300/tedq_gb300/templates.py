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


def lattice_bonds(rows, cols, layer):
    """CZ bonds of one layer of the 2-D lattice circuit: horizontal bonds on
    even layers and vertical bonds on odd layers, alternating between the two
    parity classes every second layer, so that each site takes part in at most
    one CZ per layer."""
    par = (layer // 2) % 2
    if layer % 2 == 0:
        return [(r * cols + c, r * cols + c + 1) for r in range(rows) for c in range(cols - 1) if c % 2 == par]
    return [(r * cols + c, (r + 1) * cols + c) for r in range(rows - 1) for c in range(cols) if r % 2 == par]


def lattice_params(rows, cols, layers, seed=0):
    """Haar-random SU(2) angles of every site and layer as Rot(phi, theta,
    omega): phi, omega ~ U[0, 2 pi), cos(theta) ~ U[-1, 1]; shape
    [layers * rows * cols * 3]."""
    rng = np.random.default_rng(seed)
    n = layers * rows * cols
    phi = rng.uniform(0.0, 2 * np.pi, n)
    omega = rng.uniform(0.0, 2 * np.pi, n)
    theta = np.arccos(rng.uniform(-1.0, 1.0, n))
    return np.stack([phi, theta, omega], axis=1).reshape(-1)


def lattice_spec(rows, cols, layers, params=None, seed=0, site=None):
    """2-D lattice circuit of the tensor-network workload: per layer a
    trainable Rot on every site, then CZ on the layer's bonds; one output,
    <Z> on ``site`` (default: the centre site (rows // 2, cols // 2))."""
    n = rows * cols
    if params is None:
        params = lattice_params(rows, cols, layers, seed)
    params = np.asarray(params, dtype=np.float64).reshape(layers, n, 3)
    gates = []
    for l in range(layers):
        for q in range(n):
            gates.append({"name": "Rot", "qubits": [q], "params": [float(v) for v in params[l, q]],
                          "trainable": [0, 1, 2]})
        for a, b in lattice_bonds(rows, cols, l):
            gates.append({"name": "CZ", "qubits": [a, b], "params": [], "trainable": []})
    if site is None:
        site = (rows // 2) * cols + cols // 2
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [int(site)]}]}]
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


def mbl_spec(n, layers, seed, dt=0.1, J=1.0, W=5.0):
    """1-D many-body-localisation Trotter circuit: per layer RZ(h_i dt) on every
    site (h_i ~ U[-W, W] from ``seed``) and, on every bond, RXX(J dt) =
    (H x H) CNOT RZ CNOT (H x H) and RZZ(J dt) = CNOT RZ CNOT, the
    decomposition the reference's examples use; every RZ angle is trainable;
    outputs <Z_i> on every site."""
    rng = np.random.default_rng(seed)
    h = rng.uniform(-W, W, n)
    g = []

    def add(name, q, p=None):
        g.append({"name": name, "qubits": q, "params": [] if p is None else [float(p)],
                  "trainable": [] if p is None else [0]})
    for _ in range(layers):
        for q in range(n):
            add("RZ", [q], h[q] * dt)
        for q in range(n - 1):
            add("Hadamard", [q])
            add("Hadamard", [q + 1])
            add("CNOT", [q, q + 1])
            add("RZ", [q + 1], J * dt)
            add("CNOT", [q, q + 1])
            add("Hadamard", [q])
            add("Hadamard", [q + 1])
            add("CNOT", [q, q + 1])
            add("RZ", [q + 1], J * dt)
            add("CNOT", [q, q + 1])
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n)]
    return {"n": n, "gates": g, "meas": meas, "init_state": None}
