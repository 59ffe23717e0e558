"""GPU parity of the tensor-network mode (level launches, gather kernels and the
library's GEMMs through ``tedq_tn_contract``) against the complex128 oracle of
the state-vector path and the float64 executor of the exported plan.

Tolerances: complex64 with 3xTF32 tensor-core or FP32 GEMMs within 1e-5
(expvals are bounded by 1); complex64 with single TF32 products within 5e-3;
complex128 within 1e-12.
"""

import numpy as np
import pytest
import torch

import tn_interp
from test_tn_plan import flat_params, oracle_out, random_spec

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300.templates import hea_spec, lattice_spec  # noqa: E402

DEV = "cuda:0"
TOL = {("c64", "tc32"): 1e-5, ("c64", "fp32"): 1e-5, ("c64", "auto"): 1e-5, ("c64", "tf32"): 5e-3,
       ("c128", "auto"): 1e-12}


def _tn(spec, precision="c64", gemm="fp32", **kw):
    return qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", tn_mode=True, precision=precision,
                                                      tn_gemm=gemm, **kw)


def _rdt(precision):
    return torch.float64 if precision == "c128" else torch.float32


@pytest.fixture(autouse=True)
def _native_loaded():
    yield
    assert qai._lib._lib is not None, "native library was not used"


@pytest.mark.parametrize("mode", [("c64", "tc32"), ("c64", "fp32"), ("c64", "auto"), ("c64", "tf32"),
                                  ("c128", "auto")],
                         ids=["c64-tc32", "c64-fp32", "c64-auto", "c64-tf32", "c128"])
@pytest.mark.parametrize("seed", range(6))
def test_tn_random_circuits(seed, mode):
    precision, gemm = mode
    spec = random_spec(seed)
    cc = _tn(spec, precision, gemm, requires_grad=False)
    prm = flat_params(spec)
    rng = np.random.default_rng(seed)
    rows = [prm] + [list(rng.uniform(0, 2 * np.pi, len(prm))) for _ in range(4)]
    P = torch.tensor(rows, dtype=_rdt(precision), device=DEV).reshape(len(rows), len(prm))
    got = cc.execute_batch(P).cpu().numpy()
    want = np.stack([oracle_out(spec, r) for r in rows])
    tol = TOL[mode]
    np.testing.assert_allclose(got, want, atol=tol, rtol=tol)


def test_tn_matches_state_vector_hea():
    spec = hea_spec(10, 4)
    spec["meas"] = spec["meas"][:3] + [{"kind": "expval", "list": True,
                                        "obs": [{"name": "PauliZ", "qubits": [0]}, {"name": "PauliX", "qubits": [9]}]}]
    prm = np.random.default_rng(7).uniform(0, 2 * np.pi, (16, len(flat_params(spec))))
    P = torch.tensor(prm, dtype=torch.float32, device=DEV)
    sv = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", requires_grad=False)
    tn = _tn(spec, requires_grad=False)
    np.testing.assert_allclose(tn.execute_batch(P).cpu().numpy(), sv.execute_batch(P).cpu().numpy(),
                               atol=1e-5, rtol=1e-5)


def test_tn_slicing_on_device():
    spec = random_spec(53, n=6, n_gates=40)
    prm = flat_params(spec)
    cc = _tn(spec, "c128", requires_grad=False)
    target = cc.program_info["max_rank"] - 1
    sl = _tn(spec, "c128", tn_max_rank=target, requires_grad=False)
    assert sl.program_info["n_sliced"] >= 1
    P = torch.tensor([prm], dtype=torch.float64, device=DEV)
    np.testing.assert_allclose(sl.execute_batch(P).cpu().numpy()[0], oracle_out(spec, prm), atol=1e-12, rtol=1e-12)


def test_tn_lattice_6x6_centre_z():
    """The 6x6, 8-layer workload on the device, complex64 (default GEMM mode)
    and complex128, for 5 parameter rows, against the independent
    tensor-network oracle in complex128 (oracle/tn_oracle.py: its own network
    builder and greedy order), and complex128 against the float64 plan
    executor."""
    from oracle import tn_oracle
    spec = lattice_spec(6, 6, 8, seed=0)
    prm = flat_params(spec)
    rng = np.random.default_rng(1)
    rows = np.stack([prm] + [rng.uniform(0, 2 * np.pi, len(prm)) for _ in range(4)])
    want = np.array([tn_oracle.expval(spec, torch.tensor(r, dtype=torch.float64), light_cone=True)[0]
                     for r in rows])
    c128 = _tn(spec, "c128", requires_grad=False)
    v128 = c128.execute_batch(torch.tensor(rows, dtype=torch.float64, device=DEV)).cpu().numpy()[:, 0]
    np.testing.assert_allclose(v128, want, atol=1e-12, rtol=1e-12)
    assert abs(v128[0] - tn_interp.run(c128.describe(), prm)[0]) < 1e-12
    for gemm, tol in (("auto", 1e-5), ("tc32", 1e-5), ("fp32", 1e-5), ("tf32", 5e-3)):
        c64 = _tn(spec, "c64", gemm, requires_grad=False)
        v64 = c64.execute_batch(torch.tensor(rows, dtype=torch.float32, device=DEV)).cpu().numpy()[:, 0]
        np.testing.assert_allclose(v64, want, atol=tol, rtol=tol, err_msg=gemm)


def test_tn_graph_replay_follows_parameters():
    spec = lattice_spec(3, 3, 4, seed=2)
    prm = np.asarray(flat_params(spec))
    cc = _tn(spec, "c64", tn_graphs=True, requires_grad=False)
    P = torch.tensor(np.stack([prm, prm * 0.5]), dtype=torch.float32, device=DEV)
    outs = []
    for k in range(4):  # eager, capture, replay, replay with new values in the same buffer
        if k == 3:
            P.mul_(0.25)
        outs.append(cc.execute_batch(P).cpu().numpy())
    np.testing.assert_allclose(outs[1], outs[0], atol=0, rtol=0)
    np.testing.assert_allclose(outs[2], outs[0], atol=0, rtol=0)
    want = np.stack([oracle_out(spec, r) for r in P.double().cpu().numpy()])
    np.testing.assert_allclose(outs[3], want, atol=1e-5, rtol=1e-5)


def test_tn_gradient_matches_adjoint():
    spec = random_spec(4)
    prm = flat_params(spec)
    sv = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", precision="c128")
    tn = _tn(spec, "c128")
    p1 = torch.tensor(prm, dtype=torch.float64, device=DEV, requires_grad=True)
    p2 = torch.tensor(prm, dtype=torch.float64, device=DEV, requires_grad=True)
    sv(p1).sum().backward()
    tn(p2).sum().backward()
    np.testing.assert_allclose(p2.grad.cpu().numpy(), p1.grad.cpu().numpy(), atol=1e-10, rtol=1e-10)


def test_tn_workspace_and_errors():
    spec = random_spec(2)
    cc = _tn(spec, requires_grad=False)
    prog = cc._prog
    assert prog.workspace_bytes(4096) > prog.workspace_bytes(1)
    P = torch.zeros((1, prog.n_params + 1), device=DEV)
    with pytest.raises(ValueError):
        cc.execute_batch(P)


def test_tn_level_launch_tables_follow_batch_size():
    """The item tables of the level launches (all fused steps of one
    dependency level in one kernel) are rebuilt when the batch size changes:
    calls alternating between batch sizes agree with one-circuit calls."""
    spec = hea_spec(10, 3)
    cc = _tn(spec, "c64", "fp32", requires_grad=False)
    n = len(flat_params(spec))
    gen = torch.Generator().manual_seed(4)
    P = (torch.rand(7, n, generator=gen) * 6.28).to(DEV)
    ones = torch.cat([cc.execute_batch(P[i:i + 1]) for i in range(7)])
    for rows in (3, 7, 3, 5):
        got = cc.execute_batch(P[:rows])
        torch.testing.assert_close(got, ones[:rows], atol=2e-6, rtol=1e-5)


@pytest.mark.parametrize("gemm", ["tc32", "auto", "fp32"])
def test_tn_non_finite_parameter_gives_nan(gemm):
    """A circuit with a NaN or infinite parameter returns NaN (as the
    state-vector path does); the other circuits of the batch are unaffected."""
    spec = lattice_spec(3, 3, 2, seed=1)
    cc = _tn(spec, "c64", gemm, requires_grad=False)
    n = len(flat_params(spec))
    gen = torch.Generator().manual_seed(1)
    P = (torch.rand(4, n, generator=gen) * 6.28).to(DEV)
    clean = cc.execute_batch(P)
    P[1, 0] = float("nan")
    P[2, n - 1] = float("inf")
    got = cc.execute_batch(P)
    assert torch.isnan(got[1]).all() and torch.isnan(got[2]).all()
    torch.testing.assert_close(got[[0, 3]], clean[[0, 3]], atol=1e-6, rtol=1e-5)


def test_tn_probs_match_state_vector():
    """probs(qubits=...) in the tensor-network mode (one network per outcome)
    agrees with the state-vector path, values and parameter-shift gradients.
    The tensor-network mode orders the outcome axes as the qubits are given
    (the reference's open output indices, tensor_network.py:1017-1022), the
    state-vector mode in ascending qubit order (pytorch_backend.py:461-472)."""
    spec = hea_spec(8, 3)
    spec["meas"] = [{"kind": "probs", "qubits": [5, 2]}]
    tn = _tn(spec, "c64", "fp32")
    sv = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300")
    n = len(flat_params(spec))
    gen = torch.Generator().manual_seed(7)
    P = (torch.rand(3, n, generator=gen) * 6.28).to(DEV)
    torch.testing.assert_close(tn.execute_batch(P), sv.execute_batch(P).transpose(-1, -2), atol=2e-6, rtol=1e-5)
    p1 = P[0].clone().requires_grad_(True)
    p2 = P[0].clone().requires_grad_(True)
    w = torch.arange(4, dtype=torch.float32, device=DEV).reshape(1, 2, 2)
    (tn(p1) * w).sum().backward()
    (sv(p2) * w.transpose(-1, -2)).sum().backward()
    torch.testing.assert_close(p1.grad, p2.grad, atol=2e-5, rtol=1e-4)


def test_tn_wide_probs_on_state_vector_passes():
    """probs over more than 8 qubits in the tensor-network mode are evaluated
    on the state-vector passes (2^9 or more outcome networks would be needed)
    with the tensor-network mode's outcome axes, in the given qubit order:
    values against the state-vector mode with its (ascending) axes permuted,
    and gradients through the permutation."""
    spec = hea_spec(10, 2)
    given = [9, 0, 4, 1, 8, 2, 7, 3, 6]
    spec["meas"] = [{"kind": "probs", "qubits": given}]
    tn = _tn(spec, "c64", "fp32")
    assert not tn._tn
    sv = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300")
    n = len(flat_params(spec))
    gen = torch.Generator().manual_seed(11)
    P = (torch.rand(2, n, generator=gen) * 6.28).to(DEV)
    axes = [sorted(given).index(q) for q in given]
    want = sv.execute_batch(P)[:, 0].permute([0] + [1 + a for a in axes])
    torch.testing.assert_close(tn.execute_batch(P)[:, 0], want, atol=1e-6, rtol=1e-5)
    w = torch.rand([2] * 9, generator=gen).to(DEV)
    p1 = P[0].clone().requires_grad_(True)
    p2 = P[0].clone().requires_grad_(True)
    (tn(p1)[0] * w).sum().backward()
    (sv(p2)[0].permute(axes) * w).sum().backward()
    torch.testing.assert_close(p1.grad, p2.grad, atol=1e-5, rtol=1e-4)
