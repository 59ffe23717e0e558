"""CPU checks of the tensor-network mode (no GPU): the native planner builds
the light-cone-reduced sandwich network, the contraction order, the slicing
and the gather tables on the host; ``tn_interp`` executes the exported plan
the way the device does, in float64, and the result is compared with the
complex128 oracle of the state-vector path."""

import ctypes
import time

import numpy as np
import pytest
import torch

import oracle.sv_oracle as so
import tn_interp
from conftest import load_cases

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402
from tedq_gb300.templates import lattice_spec  # noqa: E402

ONE_Q = ["Hadamard", "PauliX", "PauliY", "PauliZ", "S", "T", "SX"]
TWO_Q = ["CNOT", "CZ", "CY", "SWAP"]
THREE_Q = ["CSWAP", "Toffoli"]
PARAM_1Q = {"RX": 1, "RY": 1, "RZ": 1, "PhaseShift": 1, "Rot": 3}
PARAM_2Q = {"CRX": 1, "CRY": 1, "CRZ": 1, "ControlledPhaseShift": 1}
OBS = ["PauliX", "PauliY", "PauliZ", "Hadamard", "I"]


def random_spec(seed, n=None, n_gates=None):
    rng = np.random.default_rng(seed)
    n = n or int(rng.integers(3, 7))
    n_gates = n_gates or int(rng.integers(15, 35))
    gates = []
    for _ in range(n_gates):
        kind = rng.choice(["1q", "2q", "3q", "p1", "p2"], p=[0.2, 0.2, 0.05, 0.4, 0.15])
        if kind == "3q" and n < 3:
            kind = "2q"
        if kind == "1q":
            g = {"name": str(rng.choice(ONE_Q)), "qubits": [int(rng.integers(n))], "params": [], "trainable": []}
        elif kind == "2q":
            q = rng.choice(n, 2, replace=False)
            g = {"name": str(rng.choice(TWO_Q)), "qubits": [int(x) for x in q], "params": [], "trainable": []}
        elif kind == "3q":
            q = rng.choice(n, 3, replace=False)
            g = {"name": str(rng.choice(THREE_Q)), "qubits": [int(x) for x in q], "params": [], "trainable": []}
        else:
            table = PARAM_1Q if kind == "p1" else PARAM_2Q
            name = str(rng.choice(sorted(table)))
            k = 1 if kind == "p1" else 2
            q = rng.choice(n, k, replace=False)
            npar = table[name]
            params = [float(v) for v in rng.uniform(0, 2 * np.pi, npar)]
            # some parameters fixed (trainable_params subset), as the reference allows
            trainable = [j for j in range(npar) if rng.random() < 0.8]
            g = {"name": name, "qubits": [int(x) for x in q], "params": params, "trainable": trainable}
        if rng.random() < 0.1 and g["name"] in ("S", "T", "SX"):
            g["inv"] = True
        gates.append(g)
    meas = []
    for _ in range(int(rng.integers(1, 4))):
        k = int(rng.integers(1, min(3, n) + 1))
        q = rng.choice(n, k, replace=False)
        obs = [{"name": str(rng.choice(OBS)), "qubits": [int(x)]} for x in q]
        meas.append({"kind": "expval", "list": k > 1, "obs": obs})
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


def flat_params(spec):
    return [g["params"][t] for g in spec["gates"] for t in g["trainable"]]


def oracle_out(spec, prm):
    out = so.run(spec, torch.tensor(prm, dtype=torch.float64), torch.complex128)
    return out.reshape(-1).numpy().real


def plan(spec, **kw):
    circ = qai.Circuit.from_spec(spec)
    return circ.compilecircuit(backend="gb300", tn_mode=True, precision="c128", **kw)


@pytest.mark.parametrize("seed", range(12))
def test_tn_random_circuits_match_oracle(seed):
    spec = random_spec(seed)
    cc = plan(spec)
    desc = cc.describe()
    prm = flat_params(spec)
    assert desc["n_params"] == len(prm)
    got = tn_interp.run(desc, prm)
    np.testing.assert_allclose(got, oracle_out(spec, prm), atol=1e-12, rtol=1e-12)
    for net in desc["nets"]:
        tn_interp.check_arenas(net)
    # other parameter values through the same plan
    prm2 = list(np.random.default_rng(seed + 100).uniform(0, 2 * np.pi, len(prm)))
    np.testing.assert_allclose(tn_interp.run(desc, prm2), oracle_out(spec, prm2), atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("seed", range(4))
def test_tn_slicing_keeps_value(seed):
    spec = random_spec(seed + 50, n=6, n_gates=40)
    prm = flat_params(spec)
    d0 = plan(spec).describe()
    full = tn_interp.run(d0, prm)
    target = max(net["max_rank"] for net in d0["nets"]) - 1
    desc = plan(spec, tn_max_rank=target).describe()
    assert 1 <= max(len(net["sliced"]) for net in desc["nets"]) <= 10
    for net in desc["nets"]:
        assert net["max_rank"] <= target
        tn_interp.check_arenas(net)
    got = tn_interp.run(desc, prm)
    np.testing.assert_allclose(got, full, atol=1e-12, rtol=1e-12)
    np.testing.assert_allclose(got, oracle_out(spec, prm), atol=1e-12, rtol=1e-12)


def test_tn_golden_cases():
    done = 0
    for case in load_cases():
        if case.get("init_state") is not None or any(m["kind"] != "expval" for m in case["meas"]):
            continue
        desc = plan(case).describe()
        got = tn_interp.run(desc, case["params"])
        want = np.asarray(case["out_c128"], dtype=np.float64).reshape(-1)
        np.testing.assert_allclose(got, want, atol=1e-12, rtol=1e-12)
        done += 1
    assert done >= 3


def test_tn_lattice_matches_oracle():
    spec = lattice_spec(3, 3, 4, seed=3)
    prm = flat_params(spec)
    got = tn_interp.run(plan(spec).describe(), prm)
    np.testing.assert_allclose(got, oracle_out(spec, prm), atol=1e-12, rtol=1e-12)


def test_tn_light_cone():
    # corner site after two layers: only gates that can reach it are kept
    spec = lattice_spec(4, 4, 2, seed=1, site=0)
    desc = plan(spec).describe()
    net = desc["nets"][0]
    assert net["gates_in"] == len(spec["gates"])
    assert net["gates_kept"] < net["gates_in"] // 2
    prm = flat_params(spec)
    np.testing.assert_allclose(tn_interp.run(desc, prm), oracle_out(spec, prm), atol=1e-12, rtol=1e-12)


def test_tn_lattice_6x6_plan():
    """The 6x6, 8-layer centre-<Z> network: 207 circuit gates inside the light
    cone, an order whose largest intermediate stays small, planned in seconds."""
    spec = lattice_spec(6, 6, 8, seed=0)
    t = time.time()
    cc = plan(spec)
    took = time.time() - t
    net = cc.describe()["nets"][0]
    assert net["gates_kept"] == 207
    assert net["qubits_kept"] == 36
    assert net["max_rank"] <= 20
    assert not net["sliced"]
    assert took < 20
    tn_interp.check_arenas(net)
    info = cc.program_info
    assert info["n_params"] == 36 * 8 * 3
    assert info["workspace_per_circuit"] > 0


def test_tn_capi_rejects_probs_and_bad_input():
    L = _lib.lib()
    g = (_lib.Gate * 1)()
    g[0].op = _lib.OP["Hadamard"]
    g[0].n_qubits = 1
    g[0].qubits[0] = 0
    for j in range(3):
        g[0].param_slot[j] = -1
    m = (_lib.Meas * 1)()
    m[0].kind = _lib.MEAS_PROBS
    h = ctypes.c_void_p()
    st = L.tedq_tn_plan_create(g, 1, 2, m, 1, None, ctypes.byref(h))
    assert st == _lib.ERR_UNSUPPORTED and not h.value
    assert "expectation values" in _lib.last_error()
    F = (_lib.ObsFactor * 1)()
    F[0].obs = _lib.OBS["PauliZ"]
    F[0].n_qubits = 1
    F[0].qubits[0] = 5  # out of range
    m[0].kind = _lib.MEAS_EXPVAL
    m[0].n_factors = 1
    m[0].factors = F
    st = L.tedq_tn_plan_create(g, 1, 2, m, 1, None, ctypes.byref(h))
    assert st == _lib.ERR_ARG and not h.value
    F[0].qubits[0] = 1
    st = L.tedq_tn_plan_create(g, 1, 2, m, 1, None, ctypes.byref(h))
    assert st == _lib.OK and h.value
    assert L.tedq_tn_workspace_bytes(h, 0) < 0  # batch must be >= 1
    assert L.tedq_tn_plan_destroy(h) == _lib.OK


def test_tn_mode_state_and_wide_probs():
    """A state measurement's network keeps every output index open
    (tensor_network.py:953-955): the tensor-network mode evaluates it on the
    state-vector passes, and so are probs over more than 8 qubits (2^9 or
    more outcome networks), whose outcome axes keep the tensor-network
    convention (given qubit order)."""
    spec = random_spec(1)
    spec["meas"] = [{"kind": "state"}]
    cc = plan(spec)
    assert not cc._tn and cc._prog.has_state and cc._tn_axes
    spec = random_spec(2, n=10)
    spec["meas"] = [{"kind": "probs", "qubits": None}]  # 2^10 outcome networks
    cc = plan(spec)
    assert not cc._tn and cc._tn_axes
    spec["meas"] = [{"kind": "probs", "qubits": [9, 0, 4, 1, 8, 2, 7, 3, 6]}]
    cc = plan(spec)
    assert not cc._tn and cc._tn_axes
    spec["meas"] = [{"kind": "probs", "qubits": [9, 0, 4]}]  # 8 networks: tensor-network mode
    cc = plan(spec)
    assert cc._tn and not cc._tn_axes


@pytest.mark.parametrize("seed", range(6))
def test_tn_probs_match_oracle(seed):
    """probs(qubits=...) in the tensor-network mode: one network per outcome
    (projector products), outcome axes in the given qubit order with the first
    listed qubit as the most significant bit, as the reference's open output
    indices are ordered (tensor_network.py:1017-1022); the state-vector
    oracle's axes are in ascending qubit order."""
    spec = random_spec(seed + 40)
    n = spec["n"]
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, min(3, n) + 1))
    qs = [int(q) for q in rng.choice(n, k, replace=False)]
    spec["meas"] = [{"kind": "probs", "qubits": qs}]
    cc = plan(spec)
    desc = cc.describe()
    assert len(desc["nets"]) == 2 ** k
    prm = flat_params(spec)
    got = tn_interp.run(desc, prm)
    want = np.transpose(np.asarray(oracle_out(spec, prm)).reshape([2] * k), np.argsort(np.argsort(qs))).reshape(-1)
    np.testing.assert_allclose(got, want, atol=1e-12, rtol=1e-12)
    assert abs(got.sum() - 1.0) < 1e-12


@pytest.mark.parametrize("seed", range(4))
def test_tn_oracle_matches_state_vector_oracle(seed):
    """The CPU tensor-network restatement (full and light-cone networks) agrees
    with the state-vector oracle."""
    from oracle import tn_oracle
    spec = random_spec(seed + 20)
    prm = flat_params(spec)
    want = oracle_out(spec, prm)
    np.testing.assert_allclose(tn_oracle.expval(spec, prm), want, atol=1e-12, rtol=1e-12)
    np.testing.assert_allclose(tn_oracle.expval(spec, prm, light_cone=False), want, atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("seed", range(3))
def test_tn_lattice_6x6_8layers_matches_tn_oracle(seed):
    """The full benchmark network (6x6 sites, 8 layers, centre <Z>, 207 gates
    in the light cone): the planner's exported plan, executed as the device
    executes it, against the independent tensor-network oracle (its own
    network builder and greedy order; pinned to the reference's
    tensor-network mode by tests/golden/cases_ext.json)."""
    from oracle import tn_oracle
    spec = lattice_spec(6, 6, 8, seed=seed)
    prm = flat_params(spec)
    got = tn_interp.run(plan(spec).describe(), prm)
    want = tn_oracle.expval(spec, torch.tensor(prm, dtype=torch.float64), light_cone=True)
    np.testing.assert_allclose(got, want, atol=1e-12, rtol=1e-12)
