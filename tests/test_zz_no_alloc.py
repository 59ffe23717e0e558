"""tedq_run_noalloc: the forward entry point for callers that cannot allocate
device memory where they run circuits (inside stream capture, allocator
callbacks, real-time loops, embedders whose memory belongs to another
runtime).  Its workspace is a static device array of the library; this test
calls it through the C ABI twice in a row and compares each result with
tedq_run's on the same inputs.  The file is named to be collected last."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402

DEV = "cuda:0"


def _circuit():
    n = 12
    rng = np.random.default_rng(11)

    def circuit_def(*p):
        k = 0
        for _ in range(2):
            for q in range(n):
                qai.RY(p[k], qubits=[q]); k += 1
                qai.RZ(p[k], qubits=[q]); k += 1
            for q in range(n - 1):
                qai.CNOT(qubits=[q, q + 1])
        return [qai.probs(qubits=[0, 5]), qai.probs(qubits=[3, 11])]
    params = rng.uniform(0, 2 * np.pi, 4 * n)
    circ = qai.Circuit(circuit_def, n, *params)
    return circ.compilecircuit(backend="gb300", requires_grad=False)


def _noalloc(cc, P):
    L = _lib.lib()
    prog = cc._prog
    B = P.shape[0]
    psi = torch.empty((B, 1 << prog.ns), dtype=prog.cdtype, device=DEV)
    out = torch.empty((B, prog.n_real), dtype=prog.rdtype, device=DEV)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.tedq_run_noalloc(prog.handle, ctypes.c_void_p(P.data_ptr()), B, ctypes.c_void_p(psi.data_ptr()),
                            ctypes.c_void_p(out.data_ptr()), None, stream)
    _lib.check(st, "tedq_run_noalloc")
    torch.cuda.synchronize()
    return out, psi


def test_noalloc_matches_tedq_run_twice():
    cc = _circuit()
    gen = torch.Generator().manual_seed(5)
    for _ in range(2):
        P = (torch.rand(6, cc.num_params, generator=gen) * 2 * np.pi).to(DEV)
        ref_out, ref_psi = cc._forward(P)
        torch.cuda.synchronize()
        out, psi = _noalloc(cc, P)
        torch.testing.assert_close(out, ref_out, atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(psi, ref_psi, atol=1e-6, rtol=1e-6)


def test_noalloc_rejects_batch_beyond_static_scratch():
    cc = _circuit()
    L = _lib.lib()
    big = 1
    while cc._prog.workspace_bytes(big) <= (1 << 20):
        big *= 2
    st = L.tedq_run_noalloc(cc._prog.handle, None, big, None, None, None, None)
    assert st == _lib.ERR_ARG
    assert "static" in _lib.last_error()
