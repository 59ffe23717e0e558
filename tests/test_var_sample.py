"""``var`` and ``sample`` (declared but not implemented by the reference,
measurement.py:158-171): variance from two device expectation values, shots
drawn on the device from the probabilities in the observable's eigenbasis."""

import numpy as np
import pytest
import torch

import oracle

qai = pytest.importorskip("tedq_gb300")


def _circ(meas_fn, n=3):
    def circuit_def(*p):
        qai.RY(p[0], qubits=[0])
        qai.RX(p[1], qubits=[1])
        qai.CNOT(qubits=[0, 1])
        qai.RY(p[2], qubits=[2])
        qai.CZ(qubits=[1, 2])
        return meas_fn()

    return qai.Circuit(circuit_def, n, *torch.rand(3))


def test_recording_and_compile_without_gpu():
    c = _circ(lambda: [qai.var(qai.PauliZ(qubits=[0])), qai.var([qai.PauliX(qubits=[1]), qai.PauliZ(qubits=[2])])])
    assert [m.return_type.value for m in c.measurements] == ["var", "var"]
    cc = c.compilecircuit(backend="gb300", jit=-1)
    assert [it[0] for it in cc._prog.layout] == ["var", "var"]
    assert cc._prog.n_real == 4  # <O> and <O^2> per variance
    s = _circ(lambda: [qai.sample(qai.PauliZ(qubits=[0]), 100), qai.sample(qai.PauliX(qubits=[2]), 100)])
    cs = s.compilecircuit(backend="gb300", jit=-1, requires_grad=False)
    assert cs._sampler.qubits == [0, 2] and cs._sampler.shots == 100
    with pytest.raises(Exception):
        _circ(lambda: qai.sample(qai.PauliZ(qubits=[0]), 0))


@pytest.mark.gpu
def test_variance_values_and_gradient():
    c = _circ(lambda: [qai.var(qai.PauliZ(qubits=[0])), qai.var([qai.PauliX(qubits=[1]), qai.PauliZ(qubits=[2])])])
    cc = c.compilecircuit(backend="gb300", precision="c128")
    p = torch.tensor([0.3, 1.1, -0.7], dtype=torch.float64, requires_grad=True)
    v = cc(p)
    # Pauli products square to the identity: Var = 1 - <O>^2
    spec = oracle.spec_from_circuit(_circ(lambda: [qai.expval(qai.PauliZ(qubits=[0])),
                                                    qai.expval([qai.PauliX(qubits=[1]), qai.PauliZ(qubits=[2])])]))
    ev = oracle.run(spec, p.detach(), torch.complex128).numpy()
    np.testing.assert_allclose(v.detach().cpu().numpy(), 1 - ev ** 2, atol=1e-12)
    v.sum().backward()
    _, g_ev = oracle.value_and_grad(spec, p.detach(), -2 * ev, torch.complex128)
    np.testing.assert_allclose(p.grad.cpu().numpy(), g_ev.numpy(), atol=1e-10)


@pytest.mark.gpu
def test_sample_statistics():
    shots = 200000
    c = _circ(lambda: [qai.sample(qai.PauliZ(qubits=[0]), shots), qai.sample([qai.PauliX(qubits=[1]),
                                                                              qai.PauliY(qubits=[2])], shots)])
    cc = c.compilecircuit(backend="gb300", precision="c128", requires_grad=False)
    p = torch.tensor([0.3, 1.1, -0.7], dtype=torch.float64)
    s = cc(p).cpu().numpy()
    assert s.shape == (2, shots)
    assert set(np.unique(s)) <= {-1.0, 1.0}
    spec = oracle.spec_from_circuit(_circ(lambda: [qai.expval(qai.PauliZ(qubits=[0])),
                                                    qai.expval([qai.PauliX(qubits=[1]), qai.PauliY(qubits=[2])])]))
    ev = oracle.run(spec, p, torch.complex128).numpy()
    np.testing.assert_allclose(s.mean(axis=1), ev, atol=5 * 2 / np.sqrt(shots))
