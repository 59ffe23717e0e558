"""Dataset-parallel evaluation (the QUDIO backend's role,
qudio_backend.py:45-124): every dataset row is one circuit of a native batch."""

import numpy as np
import pytest
import torch

import oracle

qai = pytest.importorskip("tedq_gb300")


def _circuit(n=4):
    def circuit_def(x, theta):
        for i in range(n):
            qai.RY(x[i], qubits=[i])
        for i in range(n):
            qai.RZ(theta[2 * i], qubits=[i])
            qai.RX(theta[2 * i + 1], qubits=[i])
        for i in range(n - 1):
            qai.CNOT(qubits=[i, i + 1])
        return qai.probs(qubits=[n - 1])

    return qai.Circuit(circuit_def, n, torch.rand(n), torch.rand(2 * n))


def test_qudio_requires_dataset():
    circ = _circuit()
    cc = circ.compilecircuit(backend="gb300_QUDIO")
    with pytest.raises(ValueError):
        cc(torch.rand(8))


@pytest.mark.gpu
def test_qudio_rows_match_per_row_calls_and_gradients():
    n = 4
    circ = _circuit(n)
    rng = np.random.default_rng(3)
    data = torch.tensor(rng.uniform(-1, 1, (37, n)), dtype=torch.float64)
    theta = torch.tensor(rng.uniform(0, 2 * np.pi, 2 * n), dtype=torch.float64, requires_grad=True)
    qd = circ.compilecircuit(backend="gb300_QUDIO", precision="c128")
    qd.set_dataset(data)
    y = qd(theta)
    assert tuple(y.shape) == (37, 2)
    spec = oracle.spec_from_circuit(circ)
    want = np.stack([oracle.run(spec, torch.cat([data[i], theta.detach()]), torch.complex128).numpy().reshape(2)
                     for i in range(37)])
    np.testing.assert_allclose(y.detach().cpu().numpy(), want, atol=1e-12)
    # gradient of a loss over the dataset reaches theta
    y[:, 1].sum().backward()
    g = theta.grad.cpu().numpy()
    dy = np.zeros((2,))
    dy[1] = 1.0
    gsum = np.zeros(2 * n)
    for i in range(37):
        _, gi = oracle.value_and_grad(spec, torch.cat([data[i], theta.detach()]).numpy(), dy, torch.complex128)
        gsum += gi.numpy()[n:]
    np.testing.assert_allclose(g, gsum, atol=1e-10)
