"""Gradient cross-checks on the many-body-localization Trotter circuit
(RZ(h_i dt) and RXX/RZZ(J dt) decomposed as in the reference examples, all
angles trainable): the adjoint kernel against the batched parameter-shift
rule, central finite differences (eps = 1e-3) and the complex128 oracle, at
sizes the oracle finishes quickly.  Loss = sum_i <Z_i>^2."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300.templates import mbl_spec  # noqa: E402

DEV = "cuda:0"


@pytest.mark.parametrize("n,layers", [(10, 3), (12, 2)])
def test_adjoint_vs_param_shift_vs_fd_vs_oracle(n, layers):
    spec = mbl_spec(n, layers, seed=n)
    theta = np.array([gg["params"][0] for gg in spec["gates"] if gg["trainable"]])
    circ = qai.Circuit.from_spec(spec)
    # adjoint through autograd, loss = sum <Z_i>^2
    cc = circ.compilecircuit(backend="gb300", precision="c128")
    p = torch.tensor(theta, dtype=torch.float64, device=DEV).reshape(1, -1).requires_grad_(True)
    out = cc.execute_batch(p)
    (out ** 2).sum().backward()
    g_adj = p.grad[0].cpu().numpy()
    z = out[0].detach().cpu().numpy()
    # parameter shift and central differences: Jacobian of <Z_i>, chained with dL/d<Z_i> = 2<Z_i>
    P = torch.tensor(theta, dtype=torch.float64, device=DEV).reshape(1, -1)
    g_ps = (2 * z) @ cc.jacobian_param_shift(P)[0].cpu().numpy()
    g_fd = (2 * z) @ cc.finite_diff_jacobian(P, eps=1e-3)[0].cpu().numpy()
    # complex128 oracle (reference algorithm with autograd)
    _, g_ref = oracle.value_and_grad(spec, theta, 2 * z, torch.complex128)
    g_ref = g_ref.numpy()
    np.testing.assert_allclose(g_adj, g_ref, atol=1e-11)
    np.testing.assert_allclose(g_ps, g_ref, atol=1e-11)
    np.testing.assert_allclose(g_fd, g_ref, atol=1e-6)
    # the complex64 path against the same oracle
    c64 = circ.compilecircuit(backend="gb300")
    p32 = torch.tensor(theta, dtype=torch.float32, device=DEV).reshape(1, -1).requires_grad_(True)
    o32 = c64.execute_batch(p32)
    (o32 ** 2).sum().backward()
    np.testing.assert_allclose(p32.grad[0].cpu().double().numpy(), g_ref, atol=2e-5)


def test_mbl24_value_and_gradient_vs_compiled_oracle():
    """24 qubits (the config-3 state size; 2 Trotter layers keep the host side
    to seconds): the complex64 and complex128 device paths against the
    compiled complex128 CPU oracle (oracle/sv_ref.cpp: dense gates and its own
    adjoint sweep, pinned to the reference's goldens), which shares no code
    with the kernels.  Angles uniform in [0, 2 pi) and random cotangents dy
    (loss = sum_i dy_i <Z_i>) so that every gradient entry is exercised;
    values within 1e-5 (c64) and 1e-12 (c128), gradients within 5e-5 (c64:
    FP32 partial sums over 2^24 amplitudes per gate) and 1e-10 (c128)."""
    from oracle import sv_ref
    spec = mbl_spec(24, 2, seed=24)
    P = sum(1 for gg in spec["gates"] if gg["trainable"])
    theta = np.random.default_rng(24).uniform(0, 2 * np.pi, P)
    dy = np.random.default_rng(25).normal(size=24)
    want, g_want = sv_ref.value_and_grad(spec, theta, dy)
    assert np.abs(g_want).max() > 0.5  # a sensitive check, not a comparison of zeros
    circ = qai.Circuit.from_spec(spec)
    for precision, dt, vtol, gtol in (("c128", torch.float64, 1e-12, 1e-10), ("c64", torch.float32, 1e-5, 5e-5)):
        cc = circ.compilecircuit(backend="gb300", precision=precision)
        p = torch.tensor(theta, dtype=dt, device=DEV).reshape(1, -1).requires_grad_(True)
        out = cc.execute_batch(p)
        (out * torch.tensor(dy, dtype=dt, device=DEV)).sum().backward()
        np.testing.assert_allclose(out[0].detach().cpu().double().numpy(), want, atol=vtol)
        np.testing.assert_allclose(p.grad[0].cpu().double().numpy(), g_want, atol=gtol)
        del cc, out, p
        torch.cuda.empty_cache()
