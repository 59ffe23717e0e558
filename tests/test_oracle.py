"""Pins the CPU oracle against the reference's own outputs (no GPU needed).

* literal known-answer values from the reference's tests
  (test/test_pytorch_backend.py:386-584);
* golden vectors recorded from the reference by tests/golden/make_golden.py
  (forward in complex64 and complex128, back_prop and param-shift gradients).
"""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_cases

CASES = load_cases()


def _arr(v):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 2 and a.shape[1] == 2:
        return a[:, 0] + 1j * a[:, 1]
    return a


def test_reference_known_answers():
    spec = {"n": 2, "init_state": None,
            "gates": [{"name": "RX", "qubits": [0], "params": [0.54], "trainable": [0]},
                      {"name": "RY", "qubits": [0], "params": [0.12], "trainable": [0]}],
            "meas": [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [0]}]},
                     {"kind": "expval", "list": False, "obs": [{"name": "PauliX", "qubits": [1]}]}]}
    p = torch.tensor([0.54, 0.12])
    out = oracle.run(spec, p).numpy()
    # test_pytorch_backend.py:404-406
    assert np.array_equal(np.round(out, 5), np.round(np.array([0.85154057, 0.0], dtype=np.float32), 5))
    # test_pytorch_backend.py:496-503: d<Z0>/d(a, b)
    _, g = oracle.value_and_grad(spec, p, [1.0, 0.0])
    assert np.allclose(g.numpy(), [-0.5104387, -0.10267819], atol=1e-6)
    # test_pytorch_backend.py:544-553 (param-shift gives the same)
    jac = oracle.param_shift_jacobian(spec, p)
    assert np.allclose(jac[0].numpy(), [-0.5104387, -0.10267819], atol=1e-6)
    assert np.allclose(jac[1].numpy(), [0.0, 0.0], atol=1e-6)
    spec["meas"] = [{"kind": "state"}]
    st = oracle.run(spec, p).numpy().reshape(2, 2)
    # test_pytorch_backend.py:468-470
    want = np.array([[0.9620366 + 0.01599429j, 0], [0.05779156 - 0.26625147j, 0]])
    assert np.allclose(st, want, atol=1e-6)
    spec["meas"] = [{"kind": "probs", "qubits": None}]
    pr = oracle.run(spec, p).numpy().reshape(2, 2)
    # test_pytorch_backend.py:428
    assert np.allclose(pr, [[0.9257702, 0], [0.07422972, 0]], atol=1e-6)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_forward_matches_reference(case):
    p32 = torch.tensor(case["params"], dtype=torch.float32)
    out = oracle.run(case, p32, torch.complex64)
    assert list(out.shape) == case["shape"]
    np.testing.assert_allclose(out.numpy().reshape(-1), _arr(case["out_c64"]), atol=2e-6, rtol=1e-5)
    p64 = torch.tensor(case["params"], dtype=torch.float64)
    out = oracle.run(case, p64, torch.complex128)
    np.testing.assert_allclose(out.numpy().reshape(-1), _arr(case["out_c128"]), atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("case", [c for c in CASES if c["params"]], ids=[c["name"] for c in CASES if c["params"]])
def test_oracle_backprop_matches_reference(case):
    _, g = oracle.value_and_grad(case, case["params"], case["dy"], torch.complex64)
    np.testing.assert_allclose(g.numpy(), case["grad_backprop_c64"], atol=1e-5, rtol=1e-5)
    _, g = oracle.value_and_grad(case, case["params"], case["dy"], torch.complex128)
    np.testing.assert_allclose(g.numpy(), case["grad_backprop_c128"], atol=1e-11, rtol=1e-11)


PS = [c for c in CASES if "grad_paramshift_c64" in c and len(c["params"]) <= 64]


@pytest.mark.parametrize("case", PS, ids=[c["name"] for c in PS])
def test_oracle_paramshift_matches_reference(case):
    jac = oracle.param_shift_jacobian(case, case["params"], torch.complex64)
    vjp = torch.tensor(case["dy"], dtype=torch.float32) @ jac
    np.testing.assert_allclose(vjp.numpy(), case["grad_paramshift_c64"], atol=1e-5, rtol=1e-5)


def test_param_count_mismatch_raises():
    spec = CASES[0]
    with pytest.raises(ValueError, match="number of parameters are not matched"):
        oracle.run(spec, torch.tensor([0.1, 0.2, 0.3]))
