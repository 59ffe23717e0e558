"""The C-ABI library loads and exports every symbol include/tedq_gb300.h
declares; argument errors come back as status codes with a message (host-only
calls, no GPU)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402

HEADER = os.path.join(ROOT, "include", "tedq_gb300.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tedq_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = _declared()
    assert "tedq_run" in names and "tedq_run_adjoint" in names
    for name in names:
        assert hasattr(L, name), name
    assert set(names) <= set(_lib.SIGNATURES)


def test_abi_version():
    assert _lib.lib().tedq_abi_version() == _lib.ABI_VERSION


def test_bad_qubit_is_arg_error():
    L = _lib.lib()
    g = (_lib.Gate * 1)()
    g[0].op = _lib.OP["PauliX"]
    g[0].n_qubits = 1
    g[0].qubits[0] = 7
    h = ctypes.c_void_p()
    st = L.tedq_program_create(g, 1, 2, None, 0, None, ctypes.byref(h))
    assert st == _lib.ERR_ARG
    assert "out of range" in _lib.last_error()
    assert not h.value


def test_unsupported_measurement_count():
    L = _lib.lib()
    probs = (_lib.Meas * 17)()
    for m in probs:
        m.kind = _lib.MEAS_PROBS
    h = ctypes.c_void_p()
    st = L.tedq_program_create(None, 0, 3, probs, 17, None, ctypes.byref(h))
    assert st == _lib.ERR_UNSUPPORTED


def test_run_null_program_and_empty_batch():
    L = _lib.lib()
    assert L.tedq_run(None, None, 1, None, None, None, None, 0, None) == _lib.ERR_ARG
    g = (_lib.Gate * 1)()
    g[0].op = _lib.OP["Hadamard"]
    g[0].n_qubits = 1
    m = (_lib.Meas * 1)()
    m[0].kind = _lib.MEAS_STATE
    h = ctypes.c_void_p()
    assert L.tedq_program_create(g, 1, 1, m, 1, None, ctypes.byref(h)) == _lib.OK
    assert L.tedq_run(h, None, 0, None, None, None, None, 0, None) == _lib.OK
    assert L.tedq_run(h, None, 1, None, None, None, None, 0, None) == _lib.ERR_ARG
    assert L.tedq_program_workspace_bytes(h, 4) >= 0
    assert L.tedq_program_destroy(h) == _lib.OK


def test_backend_compile_errors_match_reference():
    def circuit_def(*p):
        qai.RY(p[0], qubits=[0])
        qai.RZ(p[1], qubits=[1])
        return qai.expval(qai.PauliZ(qubits=[0]))
    circ = qai.Circuit(circuit_def, 2, 0.1, 0.2)
    with pytest.raises(ValueError):
        circ.compilecircuit(backend="gb300", interface="jax")
    with pytest.raises(ValueError, match="can not use contengra"):
        circ.compilecircuit(backend="gb300", use_cotengra=True, use_jdopttn=True)
    with pytest.raises(ValueError, match="unknown backend"):
        circ.compilecircuit(backend="nope")
    cc = circ.compilecircuit(backend="gb300")
    assert cc.diff_method == "back_prop" and cc.backend == "gb300" and cc.num_params == 2
    with pytest.raises(ValueError, match="number of parameters"):
        import torch
        cc(torch.tensor([0.1, 0.2, 0.3]))


def test_specialised_kernels_compile_for_sm103a(tmp_path, monkeypatch):
    """The per-circuit kernels generated for a circuit with every gate kind
    compile with NVRTC for sm_103a (host only)."""
    monkeypatch.setenv("TEDQ_GB300_CACHE", str(tmp_path))
    from conftest import load_cases
    case = next(c for c in load_cases() if c["name"] == "all_gates_n5")
    for precision in ("c64", "c128"):
        cc = qai.Circuit.from_spec(case).compilecircuit(backend="gb300", precision=precision, jit=1)
        assert cc._prog.jit_wait() is None
    assert any(p.suffix == ".cubin" for p in tmp_path.iterdir())


@pytest.mark.parametrize("pipe", ["0", "1"])
def test_specialised_kernel_variants_compile(tmp_path, monkeypatch, pipe):
    """Both launch variants of the specialised kernels (tile pipeline and one
    tile per CTA) compile with NVRTC for sm_103a, in both precisions, for a
    circuit of several tiles per state that contains every gate kind
    (including dense phases at the start and end of passes)."""
    monkeypatch.setenv("TEDQ_GB300_CACHE", str(tmp_path))
    monkeypatch.setenv("TEDQ_GB300_PIPE", pipe)
    from conftest import load_cases
    case = dict(next(c for c in load_cases() if c["name"] == "all_gates_n5"))
    n = 15
    gates = list(case["gates"])
    for q in range(5, n):
        gates.append({"name": "RY", "qubits": [q], "params": [0.1 * q], "trainable": [0]})
        gates.append({"name": "CNOT", "qubits": [q - 1, q], "params": [], "trainable": []})
    gates += list(case["gates"])
    case.update(n=n, gates=gates)
    for precision in ("c64", "c128"):
        cc = qai.Circuit.from_spec(case).compilecircuit(backend="gb300", precision=precision, jit=1)
        for adjoint in (False, True):
            passes = cc.describe(adjoint=adjoint)["passes"]
            assert any(P["outer"] for P in passes)
            assert all(P["pipelined"] == int(pipe) for P in passes if P["outer"])
        assert cc._prog.jit_wait() is None
    assert any(p.suffix == ".cubin" for p in tmp_path.iterdir())
