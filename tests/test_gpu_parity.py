"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
vectors and the CPU oracle.

Tolerances: complex64 results within 1e-5 (absolute on expvals bounded by 1,
relative 1e-5); complex128 within 1e-12; gradients of the complex64 path
within 2e-5 of the complex128 reference.
"""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_cases

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
CASES = load_cases()
DEV = "cuda:0"


def _arr(v):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 2 and a.shape[1] == 2:
        return a[:, 0] + 1j * a[:, 1]
    return a


def _compile(case, precision, **kw):
    return qai.Circuit.from_spec(case).compilecircuit(backend="gb300", precision=precision, **kw)


def _rdt(precision):
    return torch.float64 if precision == "c128" else torch.float32


@pytest.fixture(autouse=True)
def _native_loaded():
    yield
    assert qai._lib._lib is not None, "native library was not used"


@pytest.mark.parametrize("jit", [-1, 1], ids=["generic", "specialised"])
@pytest.mark.parametrize("precision", ["c64", "c128"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_forward_matches_reference(case, precision, jit):
    cc = _compile(case, precision, jit=jit)
    if jit == 1:
        assert cc._prog.jit_wait() is None
    p = torch.tensor(case["params"], dtype=_rdt(precision), device=DEV)
    out = cc(p) if case["params"] else cc()
    assert list(out.shape) == case["shape"]
    got = out.detach().cpu().numpy().reshape(-1)
    if precision == "c64":
        np.testing.assert_allclose(got, _arr(case["out_c64"]), atol=1e-5, rtol=1e-5)
        np.testing.assert_allclose(got, _arr(case["out_c128"]), atol=1e-5, rtol=1e-5)
    else:
        np.testing.assert_allclose(got, _arr(case["out_c128"]), atol=1e-12, rtol=1e-12)


GRAD_CASES = [c for c in CASES if c["params"]]


@pytest.mark.parametrize("jit", [-1, 1], ids=["generic", "specialised"])
@pytest.mark.parametrize("precision", ["c64", "c128"])
@pytest.mark.parametrize("case", GRAD_CASES, ids=[c["name"] for c in GRAD_CASES])
def test_adjoint_grad_matches_backprop(case, precision, jit):
    cc = _compile(case, precision, jit=jit)
    p = torch.tensor(case["params"], dtype=_rdt(precision), device=DEV, requires_grad=True)
    out = cc(p)
    dy = torch.tensor(case["dy"], dtype=torch.float64, device=DEV).reshape(out.shape)
    loss = (out * dy.to(out.dtype)).real.sum() if out.is_complex() else (out * dy.to(out.dtype)).sum()
    loss.backward()
    g = p.grad.cpu().numpy()
    if precision == "c64":
        np.testing.assert_allclose(g, case["grad_backprop_c128"], atol=2e-5, rtol=2e-5)
    else:
        np.testing.assert_allclose(g, case["grad_backprop_c128"], atol=1e-11, rtol=1e-10)


PS_CASES = [c for c in CASES if "grad_paramshift_c64" in c]


@pytest.mark.parametrize("case", PS_CASES, ids=[c["name"] for c in PS_CASES])
def test_param_shift_matches_reference(case):
    cc = _compile(case, "c64", diff_method="param_shift")
    p = torch.tensor(case["params"], dtype=torch.float32, device=DEV, requires_grad=True)
    out = cc(p)
    out.backward(torch.tensor(case["dy"], dtype=torch.float32, device=DEV).reshape(out.shape))
    np.testing.assert_allclose(p.grad.cpu().numpy(), case["grad_paramshift_c64"], atol=2e-5, rtol=2e-5)


def test_reference_test_goldens_literal():
    """The values hard-coded in the reference's tests (test_pytorch_backend.py:386-553)."""
    def circuit_def(*params):
        qai.RX(params[0], qubits=[0])
        qai.RY(params[1], qubits=[0])
        return [qai.expval(qai.PauliZ(qubits=[0])), qai.expval(qai.PauliX(qubits=[1]))]
    for method in ("back_prop", "param_shift"):
        a = torch.tensor([0.54], requires_grad=True)
        b = torch.tensor([0.12], requires_grad=True)
        cc = qai.Circuit(circuit_def, 2, a, b).compilecircuit(backend="gb300", diff_method=method)
        res = cc(a, b)
        assert res.device.type == "cpu"
        assert np.array_equal(np.round(res.detach().numpy(), 5), np.round(np.array([0.85154057, 0.0], np.float32), 5))
        res[0].backward()
        assert np.round(a.grad.numpy(), 5) == np.round(np.float32(-0.5104387), 5)
        assert np.round(b.grad.numpy(), 5) == np.round(np.float32(-0.10267819), 5)


def _vqc_spec(n, layers, seed):
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers):
        for q in range(n):
            for name in ("RX", "RY", "RZ"):
                gates.append({"name": name, "qubits": [q], "params": [float(rng.uniform(0, 2 * np.pi))],
                              "trainable": [0]})
        for q in range(n - 1):
            gates.append({"name": "CNOT", "qubits": [q, q + 1], "params": [], "trainable": []})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n)]
    meas.append({"kind": "expval", "list": True,
                 "obs": [{"name": "PauliZ", "qubits": [0]}, {"name": "PauliZ", "qubits": [1]}]})
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


@pytest.mark.parametrize("jit", [-1, 1], ids=["generic", "specialised"])
@pytest.mark.parametrize("n,layers", [(14, 3), (20, 10)])
def test_batched_vqc_against_oracle(n, layers, jit):
    """Multi-pass circuits in a batch, value and adjoint gradient vs the complex128 oracle."""
    spec = _vqc_spec(n, layers, seed=n)
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=jit)
    P = cc.num_params
    gen = torch.Generator().manual_seed(n)
    params = torch.rand(3, P, generator=gen, dtype=torch.float64) * 2 * np.pi
    pd = params.to(DEV, torch.float32).requires_grad_(True)
    out = cc.execute_batch(pd)
    dy = torch.ones_like(out)
    (out * dy).sum().backward()
    for b in (0, 2):
        want, want_g = oracle.value_and_grad(spec, params[b], np.ones(out.shape[1]), torch.complex128)
        np.testing.assert_allclose(out[b].detach().cpu().double().numpy(), want.numpy(), atol=1e-5)
        np.testing.assert_allclose(pd.grad[b].cpu().double().numpy(), want_g.numpy(), atol=5e-5, rtol=1e-4)


def test_alone_equals_in_batch():
    spec = _vqc_spec(12, 2, seed=3)
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", requires_grad=False)
    params = torch.rand(8, cc.num_params, device=DEV) * 6.28
    batch = cc.execute_batch(params)
    for b in (0, 5, 7):
        alone = cc.execute_batch(params[b:b + 1])
        torch.testing.assert_close(alone[0], batch[b], atol=1e-6, rtol=1e-6)
    again = cc.execute_batch(params)
    torch.testing.assert_close(again, batch, atol=1e-7, rtol=1e-7)


@pytest.mark.parametrize("jit", [-1, 1], ids=["generic", "specialised"])
@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_gradients_alone_equal_in_batch(precision, jit):
    """The pass kernels are persistent: each CTA takes a contiguous range of
    tiles that starts and ends inside circuits, its two thread groups take
    alternate tiles, and gradient partials are flushed per circuit.  A batch
    of 37 circuits of 16 qubits (16 adjoint tiles each, about 4 per CTA) must
    give every row the values and gradients it gets alone."""
    spec = _vqc_spec(16, 2, seed=9)
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=jit, precision=precision)
    if jit == 1:
        assert cc._prog.jit_wait() is None
    rdt = _rdt(precision)
    gen = torch.Generator().manual_seed(9)
    params = (torch.rand(37, cc.num_params, generator=gen, dtype=torch.float64) * 2 * np.pi).to(DEV, rdt)
    pb = params.clone().requires_grad_(True)
    out = cc.execute_batch(pb)
    out.sum().backward()
    tol = dict(atol=1e-12, rtol=1e-12) if precision == "c128" else dict(atol=2e-6, rtol=1e-5)
    for b in (0, 1, 18, 36):
        pa = params[b:b + 1].clone().requires_grad_(True)
        alone = cc.execute_batch(pa)
        alone.sum().backward()
        torch.testing.assert_close(alone[0], out[b].detach(), **tol)
        torch.testing.assert_close(pa.grad[0], pb.grad[b], **tol)


@pytest.mark.parametrize("jit,pipe", [(-1, "0"), (1, "0"), (1, "1")],
                         ids=["generic", "specialised-one-tile", "specialised-pipelined"])
def test_zero_tile_skipping_is_exact(monkeypatch, jit, pipe):
    """Forward sweeps from |0...0> skip the tiles whose untouched qubits are
    set (all zero before and after the pass) after clearing the state: values,
    final states and adjoint gradients equal those of the same program planned
    without skipping (TEDQ_GB300_ZERO_TILES=0), in every kernel variant; a
    given initial state disables the skipping."""
    monkeypatch.setenv("TEDQ_GB300_PIPE", pipe)
    spec = _vqc_spec(16, 3, seed=4)
    circ = qai.Circuit.from_spec(spec)
    skip = circ.compilecircuit(backend="gb300", jit=jit)
    assert skip.describe()["passes"][0]["zero_outer"] != 0
    monkeypatch.setenv("TEDQ_GB300_ZERO_TILES", "0")
    full = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=jit)
    assert all(P["zero_outer"] == 0 for P in full.describe()["passes"])
    for cc in (skip, full):
        if jit == 1:
            assert cc._prog.jit_wait() is None
    gen = torch.Generator().manual_seed(4)
    params = (torch.rand(5, skip.num_params, generator=gen) * 2 * np.pi).to(DEV)
    outs, grads, states = [], [], []
    for cc in (skip, full):
        pd = params.clone().requires_grad_(True)
        out = cc.execute_batch(pd)
        out.sum().backward()
        outs.append(out.detach())
        grads.append(pd.grad)
        out_f, psi = cc._forward(params)
        states.append(psi.clone())
    # (expectation values and gradients are summed with FP64 atomics: equal
    # up to the order of those additions)
    torch.testing.assert_close(outs[0], outs[1], atol=1e-7, rtol=0)
    torch.testing.assert_close(grads[0], grads[1], atol=1e-6, rtol=1e-6)
    torch.testing.assert_close(states[0], states[1], atol=0, rtol=0)


def _unitary(k, rng):
    a = rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k))
    q, r = np.linalg.qr(a)
    u = q * (np.diag(r) / np.abs(np.diag(r)))
    return [[float(v.real), float(v.imag)] for v in u.reshape(-1)]


@pytest.mark.parametrize("jit,pipe", [(-1, "0"), (1, "0"), (1, "1")],
                         ids=["generic", "specialised-one-tile", "specialised-pipelined"])
def test_dense_phases_across_tiles(monkeypatch, jit, pipe):
    """Generic 2- and 3-qubit unitaries become dense shared-memory phases;
    placed first and last in the circuit (and between rotations) they open
    and close passes, where the pipelined kernels convert the tile between
    HBM order and pair-planar order.  15 qubits (several tiles per state),
    complex64 values and adjoint gradients against the complex128 oracle."""
    monkeypatch.setenv("TEDQ_GB300_PIPE", pipe)
    rng = np.random.default_rng(31)
    n = 15
    gates = [{"name": "Unitary", "qubits": [0, 1, 2], "params": [], "trainable": [], "matrix": _unitary(3, rng)}]
    for q in range(n):
        gates.append({"name": "RY", "qubits": [q], "params": [float(rng.uniform(0, 6.28))], "trainable": [0]})
    gates.append({"name": "Unitary", "qubits": [13, 6], "params": [], "trainable": [], "matrix": _unitary(2, rng)})
    for q in range(n - 1):
        gates.append({"name": "CNOT", "qubits": [q, q + 1], "params": [], "trainable": []})
        gates.append({"name": "RX", "qubits": [q], "params": [float(rng.uniform(0, 6.28))], "trainable": [0]})
    gates.append({"name": "Unitary", "qubits": [14, 7, 1], "params": [], "trainable": [], "matrix": _unitary(3, rng)})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(0, n, 2)]
    spec = {"n": n, "gates": gates, "meas": meas, "init_state": None}
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=jit)
    if jit == 1:
        assert cc._prog.jit_wait() is None
    dense = [ph["type"] for P in cc.describe()["passes"] + cc.describe(adjoint=True)["passes"] for ph in P["phases"]]
    assert 1 in dense
    gen = torch.Generator().manual_seed(31)
    params = torch.rand(3, cc.num_params, generator=gen, dtype=torch.float64) * 2 * np.pi
    pd = params.to(DEV, torch.float32).requires_grad_(True)
    out = cc.execute_batch(pd)
    out.sum().backward()
    for b in range(3):
        want, want_g = oracle.value_and_grad(spec, params[b], np.ones(out.shape[1]), torch.complex128)
        np.testing.assert_allclose(out[b].detach().cpu().double().numpy(), want.numpy(), atol=1e-5)
        np.testing.assert_allclose(pd.grad[b].cpu().double().numpy(), want_g.numpy(), atol=5e-5, rtol=1e-4)


def test_unfused_equals_fused():
    spec = _vqc_spec(11, 2, seed=5)
    a = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", requires_grad=False)
    b = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", requires_grad=False, fuse=False)
    params = torch.rand(4, a.num_params, device=DEV) * 6.28
    torch.testing.assert_close(a.execute_batch(params), b.execute_batch(params), atol=2e-6, rtol=1e-5)


@pytest.mark.parametrize("norm", ["0", "f", "fbu"])
@pytest.mark.parametrize("jit", [-1, 1], ids=["generic", "specialised"])
def test_register_gate_forms(monkeypatch, norm, jit):
    """Value and adjoint gradient with each choice of register-gate forms
    (plain rotations, normalised rotations in the forward passes only, and
    normalised rotations everywhere with cost-based unfusing)."""
    monkeypatch.setenv("TEDQ_GB300_NORMALISE", norm)
    spec = _vqc_spec(14, 3, seed=21)
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=jit, fuse=(norm != "f"))
    if jit == 1:
        assert cc._prog.jit_wait() is None
    gen = torch.Generator().manual_seed(21)
    # angles near 0, pi/2, pi and 3 pi / 2 select both normalised forms
    params = (torch.randint(0, 4, (2, cc.num_params), generator=gen).double() * np.pi / 2
              + 1e-3 * torch.randn(2, cc.num_params, generator=gen, dtype=torch.float64))
    pd = params.to(DEV, torch.float32).requires_grad_(True)
    out = cc.execute_batch(pd)
    out.sum().backward()
    for b in range(2):
        want, want_g = oracle.value_and_grad(spec, params[b], np.ones(out.shape[1]), torch.complex128)
        np.testing.assert_allclose(out[b].detach().cpu().double().numpy(), want.numpy(), atol=1e-5)
        np.testing.assert_allclose(pd.grad[b].cpu().double().numpy(), want_g.numpy(), atol=5e-5, rtol=1e-4)
