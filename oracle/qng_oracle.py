"""Restatement of TeD-Q's metric tensor for quantum natural gradient
(TEST INFRASTRUCTURE ONLY).

Follows tedq/QInterpreter/circuits/circuit.py: ``cycabc`` (:101-164) layers
the circuit, ``gen_circuits`` (:166-203) builds per layer the prefix circuit
plus the generators' diagonalising gates measured with ``probs`` of every
qubit, and ``metric_tensor`` / ``cov_matrix`` / ``marginal_prob``
(:297-403) form ``outer(f, f) * cov`` from marginal probabilities and the
observables' eigenvalues.  Circuits are the oracle's spec dicts; the probs come
from ``sv_oracle.run`` in complex128.
"""

import itertools

import numpy as np
import torch

from .sv_oracle import run

# generators (factor, observable) of the one-parameter gates (qubit.py:1019,
# 1077, 1134, 1295 and the controlled rotations)
_GEN = {
    "RX": (-0.5, "PauliX"), "RY": (-0.5, "PauliY"), "RZ": (-0.5, "PauliZ"),
    "PhaseShift": (1.0, np.diag([0, 1]).astype(complex)),
    "ControlledPhaseShift": (1.0, np.diag([0, 0, 0, 1]).astype(complex)),
    "CRZ": (-0.5, np.diag([0, 0, 1, -1]).astype(complex)),
}


def _generator(g):
    name = g["name"]
    if name in _GEN:
        f, o = _GEN[name]
    elif name in ("CRX", "CRY"):
        m = np.zeros((4, 4), complex)
        m[2:, 2:] = [[0, 1], [1, 0]] if name == "CRX" else [[0, -1j], [1j, 0]]
        f, o = -0.5, m
    else:
        raise ValueError(f"{name} has no generator")
    return f, (o if isinstance(o, str) else np.asarray(o)), list(g["qubits"])


def _diag_gates(obs, qubits):
    """Diagonalising gates (spec form) and eigenvalues of an observable: a
    Pauli name (PauliX -> H; PauliY -> Z, S, H; PauliZ -> none) or a matrix."""
    if isinstance(obs, str):
        names = {"PauliX": ("Hadamard",), "PauliY": ("PauliZ", "S", "Hadamard"), "PauliZ": ()}[obs]
        return ([{"name": nm, "qubits": qubits, "params": [], "trainable": []} for nm in names],
                np.array([1.0, -1.0]))
    m = np.asarray(obs)
    if np.allclose(m, np.diag(np.diag(m))):
        return [], np.diag(m).real
    vals, vecs = np.linalg.eig(m)
    d = np.linalg.inv(vecs)
    return ([{"name": "Unitary", "qubits": qubits, "params": [], "trainable": [],
              "matrix": [[float(v.real), float(v.imag)] for v in d.reshape(-1)]}], vals.real)


def layers_of(spec, numarg):
    """``cycabc`` on a spec: per layer its gates, generators and factors."""
    n = spec["n"]
    q_layers = [0] * n
    layers, obs, factors, first = {}, {}, {}, {}
    num = 0
    for g in spec["gates"]:
        ntp = len(g["trainable"])
        layer = max(q_layers[q] for q in g["qubits"])
        if ntp == 1 and num in numarg:
            f, o, qs = _generator(g)
            obs.setdefault(layer, []).append((o, qs))
            factors.setdefault(layer, []).append(f)
            first.setdefault(layer, num)
            layer += 1
        for q in g["qubits"]:
            q_layers[q] = layer
        layers.setdefault(layer, []).append((g, list(range(num, num + ntp))))
        num += ntp
    return layers, obs, factors, first


def _marginal(prob, n, axes):
    """Marginal over ``axes`` in the order given.  (The reference's
    marginal_prob keeps ascending wire order, which matches kron(l1, l2) only
    when the pair's eigenvalue vectors are symmetric or o1's wire is the lower
    one; the covariance itself is order-independent.)"""
    p = prob.reshape([2] * n)
    rest = tuple(a for a in range(n) if a not in axes)
    p = p.sum(axis=rest) if rest else p
    order = sorted(axes)
    perm = [order.index(a) for a in axes]
    return np.transpose(p, perm).reshape(-1)


def metric_tensor(spec, flat_params, numarg, reference_binding=False):
    """Block-diagonal metric tensor, float64.

    Each layer circuit's gates take the parameters they were recorded with.
    ``reference_binding=True`` restates instead what the reference's
    ``metric_tensor`` does (circuit.py:297-303): it calls the layer circuit
    with ``parameters[:num_param]`` (the first ``num_param`` flat parameters,
    ``num_param`` = index of the layer's first selected parameter), and the
    positional binding (compiled_circuit.py:492-547) hands them to the layer
    circuit's trainable gates in LAYER order (layers 0..L concatenated,
    circuit.py:181-182), which differs from gate order when unselected
    parameters or uneven layers move a gate to an earlier layer; the block is
    then evaluated at permuted parameters.  A count mismatch raises
    ``ValueError``, as the reference's binding does; a layer whose first
    selected parameter is parameter 0 is called with no parameters and keeps
    the recorded values."""
    n = spec["n"]
    flat = np.asarray(flat_params, dtype=np.float64)
    layers, obs, factors, first = layers_of(spec, set(numarg))
    blocks = []
    for L in sorted(obs):
        gates, sel = [], []
        for i in range(L + 1):
            for g, idx in layers.get(i, []):
                gates.append(g)
                sel += idx
        eig = []
        for o, qs in obs[L]:
            dg, vals = _diag_gates(o, qs)
            gates = gates + dg
            eig.append((vals, qs))
        pspec = {"n": n, "gates": gates, "meas": [{"kind": "probs", "qubits": None}], "init_state": None}
        vals = flat[sel]
        if reference_binding and first[L] > 0:
            # (a call with no parameters keeps the recorded values,
            # compiled_circuit.py:412-416)
            vals = flat[:first[L]]
            if len(vals) != len(sel):
                raise ValueError(f"Error!!!! number of parameters are not matched!! required {len(sel)} but "
                                 f"{len(vals)} are given")
        prob = run(pspec, torch.tensor(vals, dtype=torch.float64), torch.complex128)
        prob = prob.reshape(-1).numpy().real
        k = len(eig)
        cov = np.zeros((k, k))
        for i, (vals, qs) in enumerate(eig):
            p = _marginal(prob, n, qs)
            cov[i, i] = vals ** 2 @ p - (vals @ p) ** 2
        for i, j in itertools.combinations(range(k), 2):
            (v1, q1), (v2, q2) = eig[i], eig[j]
            p12 = _marginal(prob, n, q1 + q2)
            c = np.kron(v1, v2) @ p12 - (v1 @ _marginal(prob, n, q1)) * (v2 @ _marginal(prob, n, q2))
            cov[i, j] = cov[j, i] = c
        f = np.asarray(factors[L])
        blocks.append(np.outer(f, f) * cov)
    size = sum(b.shape[0] for b in blocks)
    out = np.zeros((size, size))
    k0 = 0
    for b in blocks:
        out[k0:k0 + b.shape[0], k0:k0 + b.shape[0]] = b
        k0 += b.shape[0]
    return out
