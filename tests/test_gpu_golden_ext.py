"""GPU parity against more outputs of the reference itself
(tests/golden/cases_ext.json, written by tests/golden/make_golden.py):

* the tensor-network mode (``tn_mode=True``) against the reference's own
  tensor-network branch (pytorch_backend.py:242-356): expectation values,
  ``probs`` over open output indices (given qubit order) and ``state``;
* ``states_after_measurement`` against the reference's
  (pytorch_backend.py:474-493);
* ``MetricTensor`` against the reference's ``Circuit.metric_tensor``
  (circuit.py:297-403) where the reference binds the layer circuits'
  parameters to their own gates (every parameter selected), and against the
  oracle otherwise.

Tolerances: complex64 1e-5, complex128 1e-12; the reference's metric tensor
is formed from complex64 probabilities (2e-6).
"""

import json
import os

import numpy as np
import pytest
import torch

from oracle import qng_oracle

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")

EXT = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases_ext.json")))
DEV = "cuda:0"


def _arr(v):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 2 and a.shape[1] == 2:
        return a[:, 0] + 1j * a[:, 1]
    return a


def _rdt(precision):
    return torch.float64 if precision == "c128" else torch.float32


@pytest.mark.parametrize("precision", ["c64", "c128"])
@pytest.mark.parametrize("case", EXT["tn"], ids=[c["name"] for c in EXT["tn"]])
def test_tn_mode_matches_reference_tn_branch(case, precision):
    cc = qai.Circuit.from_spec(case).compilecircuit(backend="gb300", tn_mode=True, precision=precision,
                                                    requires_grad=False)
    out = cc(torch.tensor(case["params"], dtype=_rdt(precision), device=DEV))
    assert list(out.shape) == case["shape"]
    got = out.detach().cpu().numpy().reshape(-1)
    want = _arr(case["out_c128"])
    tol = 1e-5 if precision == "c64" else 1e-12
    np.testing.assert_allclose(got, want, atol=tol, rtol=tol)


@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_states_after_measurement_match_reference(precision):
    case = EXT["after_state"][0]
    cc = qai.Circuit.from_spec(case).compilecircuit(backend="gb300", precision=precision)
    out = cc(torch.tensor(case["params"], dtype=_rdt(precision), device=DEV))
    tol = 1e-5 if precision == "c64" else 1e-12
    np.testing.assert_allclose(out.detach().cpu().numpy().reshape(-1), _arr(case["out_c128"]), atol=tol)
    after = cc.states_after_measurement
    assert sorted(after) == sorted(case["after_states_c128"])
    for key, vec in case["after_states_c128"].items():
        got = torch.stack([torch.as_tensor(x) for x in after[key]]).detach().cpu().numpy().reshape(-1)
        np.testing.assert_allclose(got, _arr(vec), atol=tol, rtol=tol)


@pytest.mark.parametrize("case", EXT["metric_tensor"], ids=[c["name"] for c in EXT["metric_tensor"]])
def test_metric_tensor_matches_reference(case):
    circ = qai.Circuit.from_spec(case)
    mt = circ.gen_circuits(case["numarg"], precision="c128")
    got = circ.metric_tensor(mt, torch.tensor(case["params"], dtype=torch.float64)).numpy()
    np.testing.assert_allclose(got, qng_oracle.metric_tensor(case, case["params"], case["numarg"]), atol=1e-12)
    if case["name"].endswith("_all"):
        np.testing.assert_allclose(got, np.asarray(case["metric_tensor"]), atol=2e-6)
