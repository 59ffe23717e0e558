"""``register_with_tedq`` on the reference's own objects (CPU; needs the
reference checkout, so it runs only where that exists).

The reference is imported unmodified (tests/golden/refshim.py).  After
registration, ``Circuit.compilecircuit(backend="gb300")`` of a circuit
recorded with the reference's own API returns a ``GB300Backend``, other
backend strings still reach the reference's method, and the C-ABI gate,
parameter-slot and measurement arrays built from the reference's circuit are
the ones built from ``tedq_gb300.Circuit.from_spec`` of the same fixture."""

import ctypes
import os
import sys

import numpy as np
import pytest
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import refshim  # noqa: E402
from conftest import load_cases  # noqa: E402

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402
from tedq_gb300.backend import GB300Backend, _Recorded  # noqa: E402

pytestmark = pytest.mark.skipif(not refshim.available(), reason="reference checkout not present")

CASES = [c for c in load_cases() if c["n"] < 14]


@pytest.fixture(scope="module")
def tq():
    mods, meta, path = set(sys.modules), list(sys.meta_path), list(sys.path)
    yield refshim.import_reference()
    for name in set(sys.modules) - mods:
        del sys.modules[name]
    sys.meta_path[:] = meta
    sys.path[:] = path


def test_register_dispatches_gb300_and_keeps_other_backends(tq):
    assert qai.register_with_tedq(tq)
    assert qai.register_with_tedq(tq)  # idempotent
    case = next(c for c in CASES if c["name"] == "hea8")
    circ = refshim.record_circuit(tq, case, torch.float32)
    cc = circ.compilecircuit(backend="gb300")
    assert isinstance(cc, GB300Backend)
    assert cc.num_params == len(case["params"])
    assert list(cc.gates_names) == [g["name"] for g in case["gates"]]
    ref = circ.compilecircuit(backend="pytorch")
    assert type(ref).__name__ == "PyTorchBackend"
    with pytest.raises(ValueError):
        circ.compilecircuit(backend="no-such-backend")


def _gate_rows(rec):
    rows = []
    for i in range(rec.n_ops):
        g = rec.gates[i]
        k = g.n_qubits
        mat = None
        if g.op == _lib.OP_MATRIX:
            mat = np.ctypeslib.as_array(g.matrix, shape=(2 * 4 ** k,)).copy()
        rows.append((g.op, k, list(g.qubits[:k]), list(g.param_slot), list(g.fixed), mat))
    return rows


def _meas_rows(rec):
    rows = []
    for i in range(rec.n_meas):
        m = rec.meas[i]
        facs = []
        for j in range(m.n_factors):
            f = m.factors[j]
            mat = None
            if f.obs == _lib.OBS_MATRIX:
                mat = np.ctypeslib.as_array(f.matrix, shape=(2 * 4 ** f.n_qubits,)).copy()
            facs.append((f.obs, f.n_qubits, list(f.qubits[:f.n_qubits]), mat))
        qs = [m.qubits[t] for t in range(m.n_qubits)] if m.n_qubits else []
        rows.append((m.kind, facs, qs))
    return rows


def _same(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return a is not None and b is not None and np.allclose(a, b, atol=1e-7)
    if isinstance(a, (list, tuple)):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    if isinstance(a, float):
        return abs(a - b) <= 1e-6 * max(1.0, abs(a))
    return a == b


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_recorded_arrays_match_from_spec(tq, case):
    ref_circ = refshim.record_circuit(tq, case, torch.float32)
    ours = qai.Circuit.from_spec(case)
    a, b = _Recorded(ref_circ), _Recorded(ours)
    assert a.n == b.n and a.n_params == b.n_params and a.n_ops == b.n_ops
    assert a.slot_of == b.slot_of
    assert [it[0] for it in a.layout] == [it[0] for it in b.layout]
    assert _same(_gate_rows(a), _gate_rows(b))
    assert _same(_meas_rows(a), _meas_rows(b))
