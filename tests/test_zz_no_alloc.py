"""tedq_run_noalloc: the forward entry point for callers that cannot allocate
device memory where they run circuits (inside stream capture, allocator
callbacks, real-time loops, embedders whose memory belongs to another
runtime).  Its workspace is a static device array of the library; it never
waits for the per-circuit kernel compile and never loads a kernel module
(which would allocate device memory for the code).

These tests call it through the C ABI, twice in a row, and compare with
tedq_run on the same inputs; a fresh 14-qubit program (specialised kernels on)
is called first through tedq_run_noalloc, which must then run the generic
kernels, load no module and still match the complex128 oracle; and a call
captured into a CUDA graph replays correctly.  The file is named to be
collected last."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402

import oracle  # noqa: E402

DEV = "cuda:0"


def _circuit(n=12, jit=0, expval=False, seed=11):
    rng = np.random.default_rng(seed)

    def circuit_def(*p):
        k = 0
        for _ in range(2):
            for q in range(n):
                qai.RY(p[k], qubits=[q]); k += 1
                qai.RZ(p[k], qubits=[q]); k += 1
            for q in range(n - 1):
                qai.CNOT(qubits=[q, q + 1])
        if expval:
            return [qai.expval(qai.PauliZ(qubits=[q])) for q in range(n)] + \
                   [qai.expval([qai.PauliX(qubits=[0]), qai.PauliY(qubits=[n - 1])])]
        return [qai.probs(qubits=[0, 5]), qai.probs(qubits=[3, 11])]
    params = rng.uniform(0, 2 * np.pi, 4 * n)
    circ = qai.Circuit(circuit_def, n, *params)
    return circ, circ.compilecircuit(backend="gb300", requires_grad=False, jit=jit)


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


def _modules_loaded(cc):
    info = _lib.ProgramInfo()
    _lib.check(_lib.lib().tedq_program_info(cc._prog.handle, ctypes.byref(info)), "tedq_program_info")
    return info.jit_modules_loaded


def test_noalloc_matches_tedq_run_twice():
    _, cc = _circuit()
    gen = torch.Generator().manual_seed(5)
    for _ in range(2):
        P = (torch.rand(6, cc.num_params, generator=gen) * 2 * np.pi).to(DEV)
        ref_out, ref_psi = cc._forward(P)
        torch.cuda.synchronize()
        out, psi = _noalloc(cc, P)
        torch.testing.assert_close(out, ref_out, atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(psi, ref_psi, atol=1e-6, rtol=1e-6)


def test_noalloc_first_call_loads_no_module():
    """A fresh program with specialised kernels: the first call is the
    allocation-free one.  It runs the generic kernels (no module loaded) and
    matches the complex128 oracle; after tedq_run has loaded the specialised
    kernels, two more calls match tedq_run."""
    circ, cc = _circuit(n=14, jit=1, expval=True, seed=3)
    assert cc.program_info["state_qubits"] >= 14
    gen = torch.Generator().manual_seed(8)
    P = torch.rand(3, cc.num_params, generator=gen, dtype=torch.float64) * 2 * np.pi
    out, _ = _noalloc(cc, P.float().to(DEV))
    assert _modules_loaded(cc) == 0
    spec = oracle.spec_from_circuit(circ)
    for b in range(P.shape[0]):
        want = oracle.run(spec, P[b], torch.complex128)
        np.testing.assert_allclose(out[b].cpu().double().numpy(), want.numpy(), atol=1e-5, rtol=0)
    for _ in range(2):
        ref_out, ref_psi = cc._forward(P.float().to(DEV))
        torch.cuda.synchronize()
        assert _modules_loaded(cc) > 0
        out2, psi2 = _noalloc(cc, P.float().to(DEV))
        torch.testing.assert_close(out2, ref_out, atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(psi2, ref_psi, atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(out2, out, atol=1e-5, rtol=1e-5)


def test_noalloc_inside_cuda_graph_capture():
    """The use the entry point exists for: a 14-qubit program with Pauli-string
    outputs (specialised kernels loaded by a warm-up tedq_run, first
    allocation-free call made before capture) is captured into a CUDA graph
    through tedq_run_noalloc; replays with new parameters written into the
    captured input buffer match tedq_run."""
    _, cc = _circuit(n=14, jit=1, expval=True, seed=5)
    assert cc._prog.jit_wait() is None
    L = _lib.lib()
    prog = cc._prog
    gen = torch.Generator().manual_seed(17)
    B = 4
    P = (torch.rand(B, cc.num_params, generator=gen) * 2 * np.pi).to(DEV)
    cc._forward(P)
    torch.cuda.synchronize()
    assert _modules_loaded(cc) > 0
    _noalloc(cc, P)
    psi = torch.empty((B, 1 << prog.ns), dtype=prog.cdtype, device=DEV)
    out = torch.empty((B, prog.n_real), dtype=prog.rdtype, device=DEV)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            st = L.tedq_run_noalloc(prog.handle, ctypes.c_void_p(P.data_ptr()), B, ctypes.c_void_p(psi.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()), None,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "tedq_run_noalloc (captured)")
    torch.cuda.current_stream().wait_stream(side)
    for _ in range(2):
        P.copy_((torch.rand(B, cc.num_params, generator=gen) * 2 * np.pi).to(DEV))
        graph.replay()
        torch.cuda.synchronize()
        ref_out, ref_psi = cc._forward(P)
        torch.cuda.synchronize()
        torch.testing.assert_close(out, ref_out, atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(psi, ref_psi, atol=1e-6, rtol=1e-6)


def test_noalloc_rejects_batch_beyond_static_scratch():
    """The limit is on the forward accumulators; the size check comes before
    any other argument is used, so null buffers are safe here."""
    _, cc = _circuit(expval=True)
    L = _lib.lib()
    big, found = 1, False
    while big <= (1 << 30):
        st = L.tedq_run_noalloc(cc._prog.handle, None, big, None, None, None, None)
        assert st == _lib.ERR_ARG
        if "static" in _lib.last_error():
            found = True
            break
        big *= 2
    assert found
    # the largest accepted power of two would not fit if the gradient region
    # (unused by the forward) were counted too
    assert cc._prog.workspace_bytes(big // 2) > (1 << 20)
