"""Pins the CPU oracles against more outputs of the reference itself
(tests/golden/cases_ext.json, written by tests/golden/make_golden.py):

* the reference's tensor-network mode (pytorch_backend.py:242-356) on
  expectation values, ``probs`` with open output indices and ``state``: the
  tensor-network oracle and the state-vector oracle give the same numbers;
* ``states_after_measurement`` (pytorch_backend.py:474-493): restated here
  from the oracle's final state;
* ``Circuit.metric_tensor`` (circuit.py:297-403): the QNG oracle.
"""

import json
import os

import numpy as np
import pytest
import torch

import oracle
from oracle import qng_oracle, tn_oracle

EXT = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cases_ext.json")))


def _arr(v):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 2 and a.shape[1] == 2:
        return a[:, 0] + 1j * a[:, 1]
    return a


TN = EXT["tn"]


@pytest.mark.parametrize("case", TN, ids=[c["name"] for c in TN])
def test_reference_tn_mode_matches_oracles(case):
    p = torch.tensor(case["params"], dtype=torch.float64)
    want128 = _arr(case["out_c128"])
    kinds = {m["kind"] for m in case["meas"]}
    if kinds == {"expval"}:
        got = tn_oracle.expval(case, p, light_cone=True)
        np.testing.assert_allclose(got, want128, atol=1e-12)
        np.testing.assert_allclose(tn_oracle.expval(case, p, light_cone=False), want128, atol=1e-12)
        sv = oracle.run(case, p, torch.complex128).numpy().reshape(-1)
    elif kinds == {"probs"}:
        # open output indices in the given qubit order; the state-vector mode
        # of the reference sorts the kept axes instead
        st = oracle.run({**case, "meas": [{"kind": "state"}]}, p, torch.complex128).numpy().reshape([2] * case["n"])
        pr = np.abs(st) ** 2
        parts = []
        for m in case["meas"]:
            qs = m["qubits"]
            rest = tuple(ax for ax in range(case["n"]) if ax not in qs)
            marg = pr.sum(axis=rest)  # axes in ascending qubit order
            parts.append(np.transpose(marg, np.argsort(np.argsort(qs))))
        sv = np.stack(parts).reshape(-1)
    else:
        sv = oracle.run(case, p, torch.complex128).numpy().reshape(-1)
    assert list(case["shape"]) == list(np.asarray(case["shape"]))
    np.testing.assert_allclose(sv, want128, atol=1e-12)
    np.testing.assert_allclose(_arr(case["out_c64"]), want128, atol=1e-5)


def test_reference_after_states_match_restatement():
    case = EXT["after_state"][0]
    p = torch.tensor(case["params"], dtype=torch.float64)
    st = oracle.run({**case, "meas": [{"kind": "state"}]}, p, torch.complex128).numpy().reshape([2] * case["n"])
    qs = case["meas"][0]["qubits"]
    assert sorted(case["after_states_c128"]) == [format(i, f"0{len(qs)}b") for i in range(2 ** len(qs))]
    for key, vec in case["after_states_c128"].items():
        sel = dict(zip(qs, (int(b) for b in key)))
        sub = st[tuple(sel.get(ax, slice(None)) for ax in range(case["n"]))]
        with np.errstate(invalid="ignore"):  # an outcome of probability 0 gives NaN, as in the reference
            sub = sub / np.sqrt(np.sum(np.abs(sub) ** 2))
        np.testing.assert_allclose(sub.reshape(-1), _arr(vec), atol=1e-12)


@pytest.mark.parametrize("case", EXT["metric_tensor"], ids=[c["name"] for c in EXT["metric_tensor"]])
def test_reference_metric_tensor_matches_qng_oracle(case):
    want = np.asarray(case["metric_tensor"])
    # the reference forms the covariances from complex64 probabilities
    got_ref = qng_oracle.metric_tensor(case, case["params"], case["numarg"], reference_binding=True)
    np.testing.assert_allclose(got_ref, want, atol=2e-6)
    got = qng_oracle.metric_tensor(case, case["params"], case["numarg"])
    if case["name"].endswith("_all"):
        # every parameter selected: layer order keeps gate order, both bindings agree
        np.testing.assert_allclose(got, want, atol=2e-6)
    else:
        # a subset moves an unselected rotation to an earlier layer: the
        # reference evaluates that block at permuted parameters
        assert np.abs(got - want).max() > 1e-3
