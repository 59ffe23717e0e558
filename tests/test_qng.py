"""Quantum natural gradient: layering on the CPU; the metric tensor on the GPU
against the restatement of the reference's per-layer probs + marginal
covariance (oracle/qng_oracle.py) and against a closed form."""

import numpy as np
import pytest
import torch

from oracle import qng_oracle

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300.qng import QNG, layer_blocks  # noqa: E402


def qng_spec(n=4, layers=3, seed=0):
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers):
        for q in range(n):
            name = ("RX", "RY", "RZ")[int(rng.integers(3))]
            gates.append({"name": name, "qubits": [q], "params": [float(rng.uniform(0, 2 * np.pi))],
                          "trainable": [0]})
        for q in range(n - 1):
            gates.append({"name": "CNOT", "qubits": [q, q + 1], "params": [], "trainable": []})
    gates.append({"name": "PhaseShift", "qubits": [1], "params": [0.3], "trainable": [0]})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [0]}]}]
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


def flat(spec):
    return [g["params"][t] for g in spec["gates"] for t in g["trainable"]]


def test_layering_matches_restatement():
    spec = qng_spec()
    circ = qai.Circuit.from_spec(spec)
    numarg = list(range(len(flat(spec))))
    layers, obs, factors, nums = layer_blocks(circ, numarg)
    ol, oo, of, on = qng_oracle.layers_of(spec, set(numarg))
    assert sorted(obs) == sorted(oo)
    for L in obs:
        assert [list(o.qubits) for o in obs[L]] == [qs for _, qs in oo[L]]
        assert factors[L] == of[L]
        assert nums[L][0] == on[L]
    assert sum(len(v) for v in layers.values()) == len(spec["gates"])


def test_multi_parameter_gate_rejected():
    spec = {"n": 1, "gates": [{"name": "Rot", "qubits": [0], "params": [0.1, 0.2, 0.3], "trainable": [0, 1, 2]}],
            "meas": [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [0]}]}],
            "init_state": None}
    with pytest.raises(ValueError):
        layer_blocks(qai.Circuit.from_spec(spec), [1])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(3))
def test_metric_tensor_matches_reference_algorithm(seed):
    spec = qng_spec(seed=seed)
    prm = flat(spec)
    numarg = list(range(len(prm)))
    circ = qai.Circuit.from_spec(spec)
    mt = circ.gen_circuits(numarg, precision="c128")
    got = circ.metric_tensor(mt, torch.tensor(prm, dtype=torch.float64)).numpy()
    want = qng_oracle.metric_tensor(spec, prm, numarg)
    np.testing.assert_allclose(got, want, atol=1e-12)
    # batched parameter vectors, complex64
    mt64 = circ.gen_circuits(numarg)
    P = torch.tensor(np.random.default_rng(seed).uniform(0, 2 * np.pi, (3, len(prm))), dtype=torch.float32)
    gb = mt64.batch(P).numpy()
    for b in range(3):
        np.testing.assert_allclose(gb[b], qng_oracle.metric_tensor(spec, P[b].double().numpy(), numarg), atol=2e-6)


@pytest.mark.gpu
def test_metric_tensor_closed_form_and_qng_step():
    """RX(a) on q0 then RY(b) on q0: g = diag(1/4, 1/4 (1 - <X>^2)) with <X> =
    0 after RX on |0>, i.e. diag(1/4, 1/4)... for RX then RY the second
    generator is measured on RX(a)|0>: Var(Y) = 1 - sin(a)^2."""
    a, b = 0.7, 0.4
    spec = {"n": 1, "gates": [{"name": "RX", "qubits": [0], "params": [a], "trainable": [0]},
                              {"name": "RY", "qubits": [0], "params": [b], "trainable": [0]}],
            "meas": [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [0]}]}],
            "init_state": None}
    circ = qai.Circuit.from_spec(spec)
    mt = circ.gen_circuits([0, 1], precision="c128")
    g = mt(torch.tensor([a, b], dtype=torch.float64)).numpy()
    # <Y> on RX(a)|0> is -sin(a)
    np.testing.assert_allclose(g, np.diag([0.25, 0.25 * (1 - np.sin(a) ** 2)]), atol=1e-12)
    # one QNG step on the expval, gradient from the adjoint backend
    cc = circ.compilecircuit(backend="gb300", precision="c128")
    x = torch.tensor([a, b], dtype=torch.float64, requires_grad=True)
    opt = QNG([x], lr=0.1)
    cc(x).sum().backward()
    grad = x.grad.clone()
    before = x.detach().clone()
    opt.step(g)
    np.testing.assert_allclose((before - x.detach()).numpy(), 0.1 * np.linalg.solve(g, grad.numpy()), atol=1e-12)
