"""Python side of the compiled complex128 state-vector oracle (TEST
INFRASTRUCTURE ONLY; oracle/sv_ref.cpp, built by oracle/build_ref.py).

``value_and_grad(spec, params, dy)`` returns the expectation values of the
spec's ``expval`` measurements and the gradient of ``sum(dy * values)`` with
respect to the flat trainable parameters, like ``sv_oracle.value_and_grad`` in
complex128, for circuits too large for the Python oracle.  Gate matrices come
from the Python oracle's restatement of the reference's gate builders
(pytorch_backend.py:579-1188), their parameter derivatives from torch autograd
on those builders; parameters are bound positionally
(compiled_circuit.py:492-547).
"""

import ctypes
import os

import numpy as np
import torch

from .sv_oracle import _gate_tensor_trainable, _matrix_from_pairs, bind_parameters, gate_matrix_fixed

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        from . import build_ref
        path = build_ref.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        L.tedq_oracle_sv_value_and_grad.restype = ctypes.c_int
        L.tedq_oracle_sv_value_and_grad.argtypes = [
            ctypes.c_int, ctypes.c_int, P(i32), P(i32), P(f64), P(i64), P(i32), P(i32), P(f64), P(i64),
            ctypes.c_int, P(i32), P(i32), P(i32), P(f64), P(i64), P(f64), ctypes.c_int, P(f64), P(f64),
            ctypes.c_int]
        _LIB = L
    return _LIB


def _pairs(m):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    return m.view(np.float64).reshape(-1)


def _gate(g, pars):
    """(matrix, [derivative matrices of the trainable parameters in order])."""
    k = len(g["qubits"])
    d = 2 ** k
    if not g["trainable"]:
        name = g["name"] + (".inv" if g.get("inv") else "")
        mat = gate_matrix_fixed(name, g["params"], g.get("matrix") and _matrix_from_pairs(g["matrix"]))
        return np.asarray(mat, dtype=np.complex128).reshape(d, d), []
    vals = [float(p.reshape(-1)[0]) if isinstance(p, torch.Tensor) else float(p) for p in pars]
    theta = torch.tensor(vals, dtype=torch.float64)

    def f(t):
        tp = [t[i:i + 1] for i in range(len(vals))]
        return torch.view_as_real(_gate_tensor_trainable(g["name"], tp, torch.complex128).reshape(d, d))

    mat = f(theta)
    jac = torch.autograd.functional.jacobian(f, theta)  # [d, d, 2, n_params_of_gate]
    dm = [(jac[..., 0, i] + 1j * jac[..., 1, i]).numpy() for i in g["trainable"]]
    return (mat[..., 0] + 1j * mat[..., 1]).numpy(), dm


def _obs_factor(o):
    mat = gate_matrix_fixed(o["name"], (), o.get("matrix") and _matrix_from_pairs(o["matrix"]))
    k = len(o["qubits"])
    return np.asarray(mat, dtype=np.complex128).reshape(2 ** k, 2 ** k)


def value_and_grad(spec, flat_params, dy=None, threads=None):
    """(values [n_expval], grad [n_params]) in float64."""
    n = spec["n"]
    if spec.get("init_state") is not None:
        raise ValueError("sv_ref: circuits start from |0...0>")
    bound = bind_parameters(spec, torch.as_tensor(np.asarray(flat_params, dtype=np.float64)), torch.float64)
    nq, qubits, mats, mat_off, n_d, d_slot, dmats, d_off = [], [], [], [], [], [], [], []
    slot, moff, doff = 0, 0, 0
    for g, pars in zip(spec["gates"], bound):
        m, dm = _gate(g, pars)
        k = len(g["qubits"])
        nq.append(k)
        qubits += list(g["qubits"]) + [0] * (3 - k)
        mat_off.append(moff)
        mats.append(_pairs(m))
        moff += 2 * m.size
        n_d.append(len(dm))
        for j, d in enumerate(dm):
            d_slot.append(slot + j)
            d_off.append(doff)
            dmats.append(_pairs(d))
            doff += 2 * d.size
        slot += len(g["trainable"])
    meas = [m for m in spec["meas"] if m["kind"] == "expval"]
    if len(meas) != len(spec["meas"]):
        raise ValueError("sv_ref: expectation values only")
    n_f, nq_f, fq, fmats, f_off = [], [], [], [], []
    foff = 0
    for m in meas:
        n_f.append(len(m["obs"]))
        for o in m["obs"]:
            fm = _obs_factor(o)
            nq_f.append(len(o["qubits"]))
            fq += list(o["qubits"]) + [0] * (3 - len(o["qubits"]))
            f_off.append(foff)
            fmats.append(_pairs(fm))
            foff += 2 * fm.size
    dyv = np.ones(len(meas)) if dy is None else np.asarray(dy, dtype=np.float64).reshape(-1)

    def arr(x, t):
        a = np.ascontiguousarray(np.asarray(x, dtype=t).reshape(-1))
        return a if a.size else np.zeros(1, dtype=t)

    A = {k: arr(v, np.int32) for k, v in (("nq", nq), ("qubits", qubits), ("n_d", n_d), ("d_slot", d_slot),
                                          ("n_f", n_f), ("nq_f", nq_f), ("fq", fq))}
    B = {k: arr(v, np.int64) for k, v in (("mat_off", mat_off), ("d_off", d_off), ("f_off", f_off))}
    C = {"mats": arr(np.concatenate(mats) if mats else [], np.float64),
         "dmats": arr(np.concatenate(dmats) if dmats else [], np.float64),
         "fmats": arr(np.concatenate(fmats) if fmats else [], np.float64), "dy": arr(dyv, np.float64)}
    values = np.zeros(max(1, len(meas)))
    grad = np.zeros(max(1, slot))

    def p(a, t):
        return a.ctypes.data_as(ctypes.POINTER(t))
    i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    rc = _lib().tedq_oracle_sv_value_and_grad(
        n, len(spec["gates"]), p(A["nq"], i32), p(A["qubits"], i32), p(C["mats"], f64), p(B["mat_off"], i64),
        p(A["n_d"], i32), p(A["d_slot"], i32), p(C["dmats"], f64), p(B["d_off"], i64), len(meas), p(A["n_f"], i32),
        p(A["nq_f"], i32), p(A["fq"], i32), p(C["fmats"], f64), p(B["f_off"], i64), p(C["dy"], f64), slot,
        p(values, f64), p(grad, f64), int(threads or os.cpu_count() or 1))
    if rc != 0:
        raise MemoryError(f"sv_ref: cannot allocate the 2^{n} state")
    return values[:len(meas)], grad[:slot]
