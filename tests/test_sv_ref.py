"""The compiled complex128 state-vector oracle (oracle/sv_ref.cpp) is pinned to
the reference's own outputs (tests/golden/cases.json: forward values and
back_prop gradients in complex128) and to the Python oracle, so that it can
check circuits too large for the Python oracle (24 qubits) on the GPU."""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_cases
from oracle import sv_ref

CASES = [c for c in load_cases() if c.get("init_state") is None and all(m["kind"] == "expval" for m in c["meas"])]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_sv_ref_matches_reference_goldens(case):
    vals, grad = sv_ref.value_and_grad(case, case["params"], case["dy"], threads=2)
    np.testing.assert_allclose(vals, np.asarray(case["out_c128"]).reshape(-1), atol=1e-12)
    if case["params"]:
        np.testing.assert_allclose(grad, case["grad_backprop_c128"], atol=1e-11)


def test_sv_ref_mbl_matches_python_oracle():
    from tedq_gb300.templates import mbl_spec
    spec = mbl_spec(10, 3, seed=5)
    P = sum(len(g["trainable"]) for g in spec["gates"])
    prm = np.random.default_rng(0).uniform(-1, 1, P)
    dy = np.random.default_rng(1).normal(size=len(spec["meas"]))
    vals, grad = sv_ref.value_and_grad(spec, prm, dy, threads=4)
    want, want_g = oracle.value_and_grad(spec, torch.tensor(prm), dy, torch.complex128)
    np.testing.assert_allclose(vals, want.numpy().reshape(-1), atol=1e-12)
    np.testing.assert_allclose(grad, want_g.numpy(), atol=1e-11)
