"""NumPy restatement of TeD-Q's tensor-network mode (TEST INFRASTRUCTURE ONLY).

The reference builds, per expectation value, the "sandwich" network
<0| U^dag O U |0> (gen_tensor_networks, tedq/tensor_network/tensor_network.py
:850-1015: zero-state vectors, the gate tensors, the observable, the mirrored
conjugate gates and the closing zero states), asks an external optimiser for a
pairwise order (opt_einsum "greedy" through OEWrapper,
tedq/oe_wrapper/oe_wrapper.py:24-65) and contracts with torch einsum
(pytorch_backend.py:242-356).  This module restates that: the same network
(optionally reduced to the backward light cone of the observable, as the
benchmark's reduced network is), a plain greedy order with opt_einsum's default
cost (size of the result minus the sizes of the inputs), and pairwise
``tensordot`` contractions in complex128 or complex64.  It is independent of
the product planner and serves as the CPU check and the CPU baseline of the
tensor-network workload.
"""

import numpy as np
import torch

from .sv_oracle import _gate_tensor_trainable, _matrix_from_pairs, bind_parameters, gate_matrix_fixed


def _gate_matrix(g, pars):
    k = len(g["qubits"])
    if len(g["trainable"]) > 0:
        tp = [p.reshape(-1)[:1].double() if isinstance(p, torch.Tensor) else torch.tensor([float(p)],
                                                                                           dtype=torch.float64)
              for p in pars]
        return _gate_tensor_trainable(g["name"], tp, torch.complex128).reshape(2 ** k, 2 ** k).numpy()
    name = g["name"] + (".inv" if g.get("inv") else "")
    return np.asarray(gate_matrix_fixed(name, g["params"], g.get("matrix") and _matrix_from_pairs(g["matrix"])),
                      dtype=np.complex128).reshape(2 ** k, 2 ** k)


def network(spec, flat_params, meas_index=0, light_cone=True):
    """Operands and index lists of the sandwich network of one expectation value.

    Returns ``(arrays, indices)``: complex128 arrays of shape (2,)*rank and,
    per array, its index labels (ints).  Ket side: |0> per qubit, then every
    gate U as a [out..., in...] tensor, then the observable factors; bra side:
    <0| per qubit and conj(U) in the same orientation; the last ket and bra
    label of each qubit coincide (tensor_network.py:995-1015 joins them
    through the observable's [out..., in...] indices the same way)."""
    n = spec["n"]
    m = spec["meas"][meas_index]
    if m["kind"] != "expval":
        raise ValueError("tensor-network oracle: expectation values only")
    bound = bind_parameters(spec, flat_params, torch.float64)
    obs = m["obs"]
    support = {q for o in obs for q in o["qubits"]}
    keep = [True] * len(spec["gates"])
    if light_cone:
        active = set(support)
        for i in range(len(spec["gates"]) - 1, -1, -1):
            qs = set(spec["gates"][i]["qubits"])
            keep[i] = bool(qs & active)
            if keep[i]:
                active |= qs
        used = active
    else:
        used = set(range(n))
    label = [0]

    def new():
        label[0] += 1
        return label[0]

    arrays, indices = [], []
    ket = {q: new() for q in sorted(used)}
    bra = {q: new() for q in sorted(used)}
    zero = np.array([1.0, 0.0], dtype=np.complex128)
    for q in sorted(used):
        arrays += [zero, zero]
        indices += [[ket[q]], [bra[q]]]

    def apply(wire, mat, qubits):
        k = len(qubits)
        ins = [wire[q] for q in qubits]
        outs = [new() for _ in qubits]
        for q, o in zip(qubits, outs):
            wire[q] = o
        arrays.append(mat.reshape([2] * (2 * k)))
        indices.append(outs + ins)

    for g, pars, kp in zip(spec["gates"], bound, keep):
        if not kp:
            continue
        mat = _gate_matrix(g, pars)
        apply(ket, mat, g["qubits"])
        apply(bra, np.conj(mat), g["qubits"])
    for o in obs:
        mat = np.asarray(gate_matrix_fixed(o["name"], (), o.get("matrix") and _matrix_from_pairs(o["matrix"])),
                         dtype=np.complex128)
        apply(ket, mat, o["qubits"])
    rename = {bra[q]: ket[q] for q in used}
    indices = [[rename.get(i, i) for i in ix] for ix in indices]
    return arrays, indices


def greedy_order(indices):
    """Pairwise order: repeatedly contract the connected pair with the lowest
    size(result) - size(a) - size(b) (opt_einsum's default greedy cost); ties
    go to the earliest pair.  Returns a list of (i, j) positions in the
    shrinking operand list, opt_einsum style (the result is appended)."""
    sets = [frozenset(ix) for ix in indices]
    order = []
    while len(sets) > 1:
        where = {}
        for t, s in enumerate(sets):
            for i in s:
                where.setdefault(i, []).append(t)
        best = None
        for ts in where.values():
            if len(ts) != 2:
                continue
            a, b = ts
            out = sets[a] ^ sets[b]
            cost = 2.0 ** len(out) - 2.0 ** len(sets[a]) - 2.0 ** len(sets[b])
            if best is None or (cost, a, b) < best:
                best = (cost, a, b)
        if best is None:  # disconnected parts: outer product of the first two
            a, b = 0, 1
        else:
            _, a, b = best
        out = sets[a] ^ sets[b]
        order.append((a, b))
        sets = [s for t, s in enumerate(sets) if t not in (a, b)] + [out]
    return order


def contract(arrays, indices, order, dtype=np.complex128):
    """Pairwise ``tensordot`` contraction along ``order``; returns the scalar."""
    ops = [np.asarray(a, dtype=dtype) for a in arrays]
    ixs = [list(ix) for ix in indices]
    for a, b in order:
        A, B, ia, ib = ops[a], ops[b], ixs[a], ixs[b]
        shared = [i for i in ia if i in ib]
        r = np.tensordot(A, B, axes=([ia.index(i) for i in shared], [ib.index(i) for i in shared]))
        out = [i for i in ia if i not in shared] + [i for i in ib if i not in shared]
        ops = [o for t, o in enumerate(ops) if t not in (a, b)] + [r]
        ixs = [x for t, x in enumerate(ixs) if t not in (a, b)] + [out]
    return complex(np.asarray(ops[0]).reshape(()))


def expval(spec, flat_params, dtype=np.complex128, light_cone=True):
    """All expectation values of ``spec`` (expval measurements only)."""
    res = []
    for m in range(len(spec["meas"])):
        arrays, indices = network(spec, flat_params, m, light_cone)
        res.append(contract(arrays, indices, greedy_order(indices), dtype).real)
    return np.array(res)
