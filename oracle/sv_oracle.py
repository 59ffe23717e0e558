"""Torch-CPU restatement of TeD-Q's state-vector execution (TEST INFRASTRUCTURE ONLY).

Every function cites the reference lines it restates (paths are inside the
TeD-Q project).  The algorithm is kept deliberately identical to the
reference's: one ``tensordot`` + ``permute`` per gate over a ``[2]*n`` tensor,
measurements by tensordot with the observable and a full contraction with the
conjugate state, gradients by torch autograd (``back_prop``) or by the
parameter-shift Jacobian.  Only the checker code (tests, smoke, the CPU legs
of the benchmark) may use it.

A circuit is described by a plain ``spec`` dict so that the same oracle can be
fed from the reference's ``Circuit`` objects, from this repository's mirror of
the circuit API, or from the JSON golden fixtures::

    {"n": int,
     "gates": [{"name": str, "qubits": [int], "params": [float],
                "trainable": [int], "inv": optional bool,
                "matrix": optional [[re, im], ...]}],
     "meas":  [{"kind": "expval", "list": bool,
                "obs": [{"name": str, "qubits": [int], "matrix": optional}]},
               {"kind": "probs", "qubits": None | [int]},
               {"kind": "state"}],
     "init_state": None | [[re, im], ...]}
"""

import cmath
import math

import numpy as np
import torch

# Gate arity / parameter counts, tedq/QInterpreter/operators/qubit.py
# (``_num_qubits`` / ``_num_params`` class attributes, lines 65-1714).
GATE_ARITY = {
    "I": 1, "Hadamard": 1, "PauliX": 1, "PauliY": 1, "PauliZ": 1, "S": 1, "T": 1, "SX": 1,
    "CNOT": 2, "CZ": 2, "CY": 2, "SWAP": 2, "CSWAP": 3, "Toffoli": 3,
    "RX": 1, "RY": 1, "RZ": 1, "Rot": 1, "PhaseShift": 1,
    "ControlledPhaseShift": 2, "CRX": 2, "CRY": 2, "CRZ": 2,
}
GATE_NPARAMS = {
    "I": 0, "Hadamard": 0, "PauliX": 0, "PauliY": 0, "PauliZ": 0, "S": 0, "T": 0, "SX": 0,
    "CNOT": 0, "CZ": 0, "CY": 0, "SWAP": 0, "CSWAP": 0, "Toffoli": 0,
    "RX": 1, "RY": 1, "RZ": 1, "Rot": 3, "PhaseShift": 1,
    "ControlledPhaseShift": 1, "CRX": 1, "CRY": 1, "CRZ": 1,
}

_INV_SQRT2 = 1.0 / math.sqrt(2.0)


def gate_matrix_fixed(name, params=(), matrix=None):
    """Record-time complex128 matrix of a gate (qubit.py ``get_matrix``).

    Restates qubit.py:68-71 (Hadamard), 152-155 (PauliX), 236-239 (PauliY),
    324-327 (PauliZ), 404-407 (I), 467-470 (S), 527-530 (T), 587-590 (SX),
    656-659 (CNOT), 705-708 (CZ), 754-757 (CY), 817-820 (SWAP), 870-885
    (CSWAP), 932-947 (Toffoli), 990-997 (RX), 1048-1055 (RY), 1106-1112
    (RZ), 1169-1189 (Rot), 1253-1257 (PhaseShift), 1327-1334
    (ControlledPhaseShift), 1429-1436 (CRX), 1531-1538 (CRY), 1631-1642
    (CRZ).  A ``.inv`` suffix is the conjugate transpose (ops_abc.py:314-323).
    """
    if name.endswith(".inv"):
        return gate_matrix_fixed(name[:-4], params, matrix).conj().T
    if matrix is not None:
        return np.asarray(matrix, dtype=np.complex128)
    p = [float(x) for x in params]
    if name == "I":
        return np.eye(2, dtype=np.complex128)
    if name == "Hadamard":
        return np.array([[_INV_SQRT2, _INV_SQRT2], [_INV_SQRT2, -_INV_SQRT2]], dtype=np.complex128)
    if name == "PauliX":
        return np.array([[0, 1], [1, 0]], dtype=np.complex128)
    if name == "PauliY":
        return np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    if name == "PauliZ":
        return np.array([[1, 0], [0, -1]], dtype=np.complex128)
    if name == "S":
        return np.array([[1, 0], [0, 1j]], dtype=np.complex128)
    if name == "T":
        return np.array([[1, 0], [0, cmath.exp(1j * np.pi / 4)]], dtype=np.complex128)
    if name == "SX":
        return 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]], dtype=np.complex128)
    if name == "CNOT":
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = [[0, 1], [1, 0]]
        return m
    if name == "CZ":
        return np.diag([1, 1, 1, -1]).astype(np.complex128)
    if name == "CY":
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = [[0, -1j], [1j, 0]]
        return m
    if name == "SWAP":
        return np.eye(4, dtype=np.complex128)[[0, 2, 1, 3]]
    if name == "CSWAP":
        return np.eye(8, dtype=np.complex128)[[0, 1, 2, 3, 4, 6, 5, 7]]
    if name == "Toffoli":
        return np.eye(8, dtype=np.complex128)[[0, 1, 2, 3, 4, 5, 7, 6]]
    if name == "RX":
        c, js = math.cos(p[0] / 2), 1j * math.sin(-p[0] / 2)
        return np.array([[c, js], [js, c]], dtype=np.complex128)
    if name == "RY":
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)
    if name == "RZ":
        e = cmath.exp(-0.5j * p[0])
        return np.array([[e, 0], [0, e.conjugate()]], dtype=np.complex128)
    if name == "Rot":
        phi, theta, omega = p
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return np.array([[cmath.exp(-0.5j * (phi + omega)) * c, -cmath.exp(0.5j * (phi - omega)) * s],
                         [cmath.exp(-0.5j * (phi - omega)) * s, cmath.exp(0.5j * (phi + omega)) * c]],
                        dtype=np.complex128)
    if name == "PhaseShift":
        return np.array([[1, 0], [0, cmath.exp(1j * p[0])]], dtype=np.complex128)
    if name == "ControlledPhaseShift":
        return np.diag([1, 1, 1, cmath.exp(1j * p[0])]).astype(np.complex128)
    if name == "CRX":
        c, js = math.cos(p[0] / 2), 1j * math.sin(-p[0] / 2)
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = [[c, js], [js, c]]
        return m
    if name == "CRY":
        c, s = math.cos(p[0] / 2), math.sin(p[0] / 2)
        m = np.eye(4, dtype=np.complex128)
        m[2:, 2:] = [[c, -s], [s, c]]
        return m
    if name == "CRZ":
        return np.diag([1, 1, cmath.exp(-0.5j * p[0]), cmath.exp(0.5j * p[0])]).astype(np.complex128)
    raise ValueError(f"oracle: unknown gate {name}")


def _as_param(x, rdtype):
    if isinstance(x, torch.Tensor):
        return x.reshape(-1)[:1] if x.dim() > 0 else x.reshape(1)
    return torch.tensor([float(x)], dtype=rdtype)


def _gate_tensor_trainable(name, pars, cdtype):
    """Call-time gate tensor of a gate with trainable parameters.

    Restates pytorch_backend.py:866-1188 (``get_RX_tensor`` ...
    ``get_CRZ_tensor``): entries built from 1-element real tensors with
    torch.cos/sin/exp, concatenated and cast to the complex dtype.
    """
    one = torch.ones(1, dtype=cdtype)
    zero = torch.zeros(1, dtype=cdtype)
    if name == "RX":
        c = torch.cos(pars[0] / 2.0)
        js = 1j * torch.sin(-pars[0] / 2.0)
        data = [c, js, js, c]
        shape = [2, 2]
    elif name == "RY":
        c = torch.cos(pars[0] / 2.0)
        s = torch.sin(pars[0] / 2.0)
        data = [c, -s, s, c]
        shape = [2, 2]
    elif name == "RZ":
        e = torch.exp(-0.5j * pars[0])
        data = [e, zero, zero, e.conj_physical()]
        shape = [2, 2]
    elif name == "Rot":
        phi, theta, omega = pars
        c = torch.cos(theta / 2.0)
        s = torch.sin(theta / 2.0)
        data = [torch.exp(-0.5j * (phi + omega)) * c, -torch.exp(0.5j * (phi - omega)) * s,
                torch.exp(-0.5j * (phi - omega)) * s, torch.exp(0.5j * (phi + omega)) * c]
        shape = [2, 2]
    elif name == "PhaseShift":
        data = [one, zero, zero, torch.exp(1.0j * pars[0])]
        shape = [2, 2]
    elif name in ("ControlledPhaseShift", "CRX", "CRY", "CRZ"):
        if name == "ControlledPhaseShift":
            blk = [one, zero, zero, torch.exp(1.0j * pars[0])]
        elif name == "CRX":
            c = torch.cos(pars[0] / 2.0)
            js = 1.0j * torch.sin(-pars[0] / 2.0)
            blk = [c, js, js, c]
        elif name == "CRY":
            c = torch.cos(pars[0] / 2.0)
            s = torch.sin(pars[0] / 2.0)
            blk = [c, -s, s, c]
        else:
            blk = [torch.exp(-0.5j * pars[0]), zero, zero, torch.exp(0.5j * pars[0])]
        data = [one, zero, zero, zero, zero, one, zero, zero,
                zero, zero, blk[0], blk[1], zero, zero, blk[2], blk[3]]
        shape = [2, 2, 2, 2]
    else:
        raise ValueError(f"oracle: gate {name} has no trainable form")
    data = [d.to(cdtype) for d in data]
    return torch.cat(data, dim=0).reshape(shape)


def spec_from_circuit(circuit):
    """Neutral description of a recorded circuit (duck-typed).

    Reads the same attributes the reference's ``CompiledCircuit.__init__``
    reads (compiled_circuit.py:82-93): per operator ``name``, ``qubits``,
    ``parameters``, ``trainable_params``, ``matrix``; the measurement list and
    the optional prepared initial state.
    """
    gates = []
    for op in circuit.operators:
        inv = op.name.endswith(".inv")
        g = {"name": op.name[:-4] if inv else op.name, "inv": inv,
             "qubits": [int(q) for q in op.qubits],
             "params": [float(p.detach().reshape(-1)[0]) if isinstance(p, torch.Tensor) else float(p)
                        for p in op.parameters],
             "trainable": [int(t) for t in op.trainable_params]}
        if g["name"] not in GATE_ARITY:
            m = np.asarray(op.matrix, dtype=np.complex128)
            g["matrix"] = [[float(v.real), float(v.imag)] for v in m.reshape(-1)]
        gates.append(g)
    meas = []
    for m in circuit.measurements:
        kind = m.return_type.value if hasattr(m.return_type, "value") else str(m.return_type)
        if kind == "expval":
            obs_list = m.obs if isinstance(m.obs, list) else [m.obs]
            obs = []
            for ob in obs_list:
                o = {"name": ob.name, "qubits": [int(q) for q in ob.qubits]}
                if ob.name not in ("I", "Hadamard", "PauliX", "PauliY", "PauliZ"):
                    mm = np.asarray(ob.matrix, dtype=np.complex128)
                    o["matrix"] = [[float(v.real), float(v.imag)] for v in mm.reshape(-1)]
                obs.append(o)
            meas.append({"kind": "expval", "list": isinstance(m.obs, list), "obs": obs})
        elif kind == "probs":
            meas.append({"kind": "probs", "qubits": None if m.qubits is None else [int(q) for q in m.qubits]})
        elif kind == "state":
            meas.append({"kind": "state"})
        else:
            raise ValueError(f"oracle: unsupported measurement {kind}")
    init = None
    if getattr(circuit, "init_state", None) is not None:
        v = np.asarray(circuit.init_state.matrix, dtype=np.complex128).reshape(-1)
        init = [[float(x.real), float(x.imag)] for x in v]
    return {"n": int(circuit.num_qubits), "gates": gates, "meas": meas, "init_state": init}


def _matrix_from_pairs(pairs):
    a = np.asarray(pairs, dtype=np.float64)
    v = a[:, 0] + 1j * a[:, 1]
    k = int(round(math.sqrt(v.size)))
    return v.reshape(k, k)


def bind_parameters(spec, flat_params, rdtype=torch.float32):
    """Per-gate parameter lists after positional binding.

    Restates compiled_circuit.py:492-547 (``_update_parameters``) together with
    pytorch_backend.py:233-239: every input is flattened to 1-element rows and
    the k-th row is assigned to the k-th trainable slot, walking the gates in
    circuit order and, inside a gate, its ``trainable_params`` list.
    """
    if isinstance(flat_params, torch.Tensor):
        rows = list(flat_params.reshape(-1, 1))
    else:
        rows = []
        for p in flat_params:
            if isinstance(p, torch.Tensor):
                rows.extend(list(p.reshape(-1, 1)))
            else:
                rows.append(torch.tensor([float(p)], dtype=rdtype))
    count = 0
    bound = []
    for g in spec["gates"]:
        pars = list(g["params"])
        for i, pos in enumerate(g["trainable"]):
            if count + i < len(rows):
                pars[pos] = rows[count + i]
        count += len(g["trainable"])
        bound.append(pars)
    if len(rows) != count:
        raise ValueError(f"Error!!!! number of parameters are not matched!! required {count} but {len(rows)} are given")
    return bound


def _apply(state, gate, qubits, n):
    """``tensordot`` + inverse permutation of one gate.

    Restates compiled_circuit.py:126-202 (axes ``gate_pos``/``state_pos`` and
    the permutation that moves the gate's output axes back to the qubit
    positions) and the loop body pytorch_backend.py:365-379.
    """
    k = len(qubits)
    gate_pos = list(range(k, 2 * k))
    new = torch.tensordot(gate, state, (gate_pos, list(qubits)))
    rest = [x for x in range(n) if x not in qubits]
    dot_result = list(qubits) + rest
    perms = [dot_result.index(i) for i in range(n)]
    return new.permute(perms)


def _obs_tensor(ob, cdtype):
    mat = gate_matrix_fixed(ob["name"], (), ob.get("matrix") and _matrix_from_pairs(ob["matrix"]))
    k = len(ob["qubits"])
    return torch.from_numpy(mat).to(cdtype).reshape([2] * (2 * k))


def run(spec, flat_params, cdtype=torch.complex64):
    """Forward pass; returns ``torch.stack`` of the measurement results.

    Restates ``PyTorchBackend.execute`` state-vector branch
    (pytorch_backend.py:358-391), ``get_initstate``/``default_initstate``
    (:500-522) and ``get_measurement_results`` (:393-498).
    """
    n = spec["n"]
    rdtype = torch.float64 if cdtype == torch.complex128 else torch.float32
    bound = bind_parameters(spec, flat_params, rdtype)
    # gate tensors, pytorch_backend.py _parser_circuit (compiled_circuit.py:418-440)
    tensors = []
    for g, pars in zip(spec["gates"], bound):
        if len(g["trainable"]) > 0:
            tp = [_as_param(x, rdtype) for x in pars]
            ts = _gate_tensor_trainable(g["name"], tp, cdtype)
        else:
            name = g["name"] + (".inv" if g.get("inv") else "")
            mat = gate_matrix_fixed(name, g["params"],
                                    g.get("matrix") and _matrix_from_pairs(g["matrix"]))
            ts = torch.from_numpy(np.ascontiguousarray(mat)).to(cdtype).reshape([2] * (2 * len(g["qubits"])))
        tensors.append(ts)
    if spec.get("init_state") is not None:
        a = np.asarray(spec["init_state"], dtype=np.float64)
        state = torch.from_numpy(a[:, 0] + 1j * a[:, 1]).to(cdtype).reshape([2] * n)
    else:
        state = torch.zeros([2] * n, dtype=cdtype)
        state.view(-1)[0] = 1.0
    for g, ts in zip(spec["gates"], tensors):
        state = _apply(state, ts, g["qubits"], n)
    results = []
    axes = list(range(n))
    for m in spec["meas"]:
        if m["kind"] == "expval":
            ms = state
            for ob in m["obs"]:
                ms = _apply(ms, _obs_tensor(ob, cdtype), ob["qubits"], n)
            r = torch.tensordot(torch.conj(state), ms, dims=(axes, axes))
            results.append(torch.squeeze(r.real))
        elif m["kind"] == "probs":
            p = torch.abs(state) ** 2
            if m["qubits"] is None:
                results.append(p)
            else:
                other = [x for x in axes if x not in m["qubits"]]
                results.append(torch.sum(p, dim=other) if other else p)
        elif m["kind"] == "state":
            results.append(state)
    return torch.stack(results, 0)


_SHIFT = np.pi / 2.0
_DEFAULT_RECIPE = [[0.5 / np.sin(_SHIFT), 1.0, _SHIFT], [-0.5 / np.sin(_SHIFT), 1.0, -_SHIFT]]
_M1 = _INV_SQRT2 * (np.sqrt(2) + 1) / 4
_M2 = _INV_SQRT2 * (np.sqrt(2) - 1) / 4
_CONTROL_RECIPE = [[_M1, 1.0, np.pi / 2], [-_M1, 1.0, -np.pi / 2],
                   [-_M2, 1.0, 3 * np.pi / 2], [_M2, 1.0, -3 * np.pi / 2]]


def shift_recipe(name):
    """Parameter-shift recipe of a gate.

    Two-term default (ops_abc.py:261-280) or the four-term controlled-rotation
    recipe (qubit.py:32-42, used by CRX/CRY/CRZ at qubit.py:1415-1427,
    1517-1529, 1617-1629).
    """
    return _CONTROL_RECIPE if name in ("CRX", "CRY", "CRZ") else _DEFAULT_RECIPE


def param_shift_jacobian(spec, flat_params, cdtype=torch.complex64):
    """Jacobian ``[len(out), P]`` by re-execution with shifted parameters.

    Restates ``jacobian_param_shift`` (pytorch_backend.py:180-212): for every
    trainable slot and every recipe term ``(c, a, s)``, all parameters are
    multiplied by ``a`` and the slot is shifted by ``s``.
    """
    rdtype = torch.float64 if cdtype == torch.complex128 else torch.float32
    params = torch.as_tensor(flat_params, dtype=rdtype).reshape(-1).detach()
    cols = []
    count = 0
    for g in spec["gates"]:
        for j in range(len(g["trainable"])):
            grad = 0.0
            for c, a, s in shift_recipe(g["name"]):
                newp = a * params.clone()
                newp[count + j] += s
                grad = grad + c * run(spec, newp, cdtype)
            cols.append(grad)
        count += len(g["trainable"])
    if not cols:
        return torch.zeros((0, 0), dtype=rdtype)
    return torch.stack([c.reshape(-1) for c in cols], dim=1)


def value_and_grad(spec, flat_params, dy, cdtype=torch.complex64):
    """Outputs and ``d(sum(dy * out))/d params`` through torch autograd.

    This is the reference's default ``back_prop`` differentiation
    (pytorch_backend.py:142-144): reverse-mode AD through the gate loop.
    """
    rdtype = torch.float64 if cdtype == torch.complex128 else torch.float32
    p = torch.as_tensor(flat_params, dtype=rdtype).reshape(-1).detach().clone().requires_grad_(True)
    out = run(spec, p, cdtype)
    dyt = torch.as_tensor(dy, dtype=torch.float64).to(out.dtype).reshape(out.shape)
    loss = (out * dyt).real.sum() if out.is_complex() else (out * dyt).sum()
    loss.backward()
    return out.detach(), p.grad.detach()


def pauli_expval_from_state(state, n, xmask, zmask):
    """Expectation of a Pauli string on a flat state (helper for checks).

    ``xmask``/``zmask`` use the flat-index bit convention of the reference:
    qubit q is bit (n-1-q) (pytorch_backend.py:513-522).
    """
    idx = np.arange(1 << n)
    psi = np.asarray(state).reshape(-1)
    flipped = psi[idx ^ xmask]
    ny = bin(xmask & zmask).count("1")
    sign = 1 - 2 * (np.vectorize(lambda v: bin(v).count("1") & 1)(idx & zmask))
    return float(np.real(np.sum(np.conj(psi) * (-1j) ** ny * sign * flipped)))
