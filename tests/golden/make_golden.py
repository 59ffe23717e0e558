"""Generate golden vectors by running the reference TeD-Q itself.

Run in a container where the reference checkout is available::

    python tests/golden/make_golden.py [/path/to/reference]

It imports the unmodified reference (``tedq``) with stub modules for its
optional dependencies that are not installed (jax, qiskit, quafu, matplotlib,
panel, IPython, toolz, ray, cotengra), records a set of seeded circuits with
the reference's own circuit API, runs them through the reference's
``PyTorchBackend`` and writes ``cases.json`` next to this script:

* forward outputs in complex64 (the reference default) and in complex128
  (module global ``tcomplex`` switched, float64 parameters);
* ``back_prop`` gradients of ``sum(dy * out)`` (``Re`` for complex outputs);
* ``param_shift`` gradients for circuits whose output is a 1-D expval list.

The fixtures are consumed by ``tests/`` on machines without the reference.

A second file, ``cases_ext.json``, records three more outputs of the
reference:

* its tensor-network mode (pytorch_backend.py:242-356, the ``use_jdopttn``
  branch with ``tn_simplify=False``) on expectation values, ``probs`` with
  open output indices and ``state``, in complex64 and complex128, with
  ``OEGreedy`` -- opt_einsum's greedy path and pairwise contraction -- in the
  place of the external JDtensorPath optimiser, which is not vendored;
* ``states_after_measurement`` after ``probs(qubits, after_state=True)``
  (pytorch_backend.py:474-493, tools/helpers.py:22-50);
* ``Circuit.metric_tensor(Circuit.gen_circuits(numarg), *params)``
  (circuit.py:166-203, 297-403) on two circuits.
"""

import json
import math
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import refshim  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else refshim.DEFAULT_PATH
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cases.json")
OUT_EXT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cases_ext.json")

qai = refshim.import_reference(REF)
import tedq.backends.pytorch_backend as pb  # noqa: E402

ONE_Q = ["Hadamard", "PauliX", "PauliY", "PauliZ", "I", "S", "T", "SX"]
TWO_Q = ["CNOT", "CZ", "CY", "SWAP"]
THREE_Q = ["CSWAP", "Toffoli"]
ROT1 = ["RX", "RY", "RZ", "PhaseShift"]
ROT2 = ["ControlledPhaseShift", "CRX", "CRY", "CRZ"]


def g(name, qubits, params=(), trainable=None, inv=False):
    d = {"name": name, "qubits": list(qubits), "params": [float(p) for p in params],
         "trainable": list(range(len(params))) if trainable is None else list(trainable)}
    if inv:
        d["inv"] = True
    return d


def expval(*obs, as_list=None):
    obs = [{"name": o[0], "qubits": list(o[1])} for o in obs]
    return {"kind": "expval", "list": (len(obs) > 1) if as_list is None else as_list, "obs": obs}


# --------------------------------------------------------------------------- cases

def case_reference_tests():
    """The circuits of the reference's own golden tests (test_pytorch_backend.py:386-584)."""
    gates = [g("RX", [0], [0.54]), g("RY", [0], [0.12])]
    return [
        ("ref_expval", 2, gates, [expval(("PauliZ", [0])), expval(("PauliX", [1]))]),
        ("ref_probs", 2, gates, [{"kind": "probs", "qubits": None}]),
        ("ref_partial_probs", 2, gates, [{"kind": "probs", "qubits": [1]}]),
        ("ref_state", 2, gates, [{"kind": "state"}]),
    ]


def case_all_gates(rng, n=4, depth=3):
    gates = []
    for _ in range(depth):
        for name in ONE_Q + ROT1 + ["Rot"]:
            q = int(rng.integers(n))
            if name == "Rot":
                gates.append(g(name, [q], rng.uniform(0, 2 * np.pi, 3)))
            elif name in ROT1:
                gates.append(g(name, [q], [rng.uniform(0, 2 * np.pi)]))
            else:
                gates.append(g(name, [q]))
        for name in TWO_Q + ROT2:
            q = [int(x) for x in rng.permutation(n)[:2]]
            gates.append(g(name, q, [rng.uniform(0, 2 * np.pi)] if name in ROT2 else []))
        for name in THREE_Q:
            q = [int(x) for x in rng.permutation(n)[:3]]
            gates.append(g(name, q))
    meas = [expval(("PauliZ", [0])), expval(("PauliX", [1])), expval(("PauliY", [2])),
            expval(("Hadamard", [3])), expval(("I", [1])),
            expval(("PauliZ", [0]), ("PauliZ", [1])),
            expval(("PauliX", [0]), ("PauliY", [2]), ("PauliZ", [3])),
            expval(("Hadamard", [1]), ("PauliX", [2]))]
    return gates, meas


def case_hea(n=8, layers=4):
    """8-qubit hardware-efficient ansatz: RY, RZ per qubit then a CNOT ring."""
    gates = []
    for _ in range(layers):
        for q in range(n):
            gates.append(g("RY", [q], [0.0]))
            gates.append(g("RZ", [q], [0.0]))
        for q in range(n):
            gates.append(g("CNOT", [q, (q + 1) % n]))
    return gates, [expval(("PauliZ", [q])) for q in range(n)]


def case_vqc(n, layers):
    """RX, RY, RZ per qubit then a CNOT ladder; outputs <Z_i> and <Z_0 Z_1>."""
    gates = []
    for _ in range(layers):
        for q in range(n):
            for name in ("RX", "RY", "RZ"):
                gates.append(g(name, [q], [0.0]))
        for q in range(n - 1):
            gates.append(g("CNOT", [q, q + 1]))
    meas = [expval(("PauliZ", [q])) for q in range(n)] + [expval(("PauliZ", [0]), ("PauliZ", [1]))]
    return gates, meas


def case_mbl(rng, n, layers, dt=0.1, J=1.0, W=5.0):
    """Trotterised MBL chain: RZ(h_i dt), RXX(J dt), RZZ(J dt) with the
    decompositions the reference examples use (H.H CNOT RZ CNOT H.H and
    CNOT RZ CNOT), all angles trainable."""
    h = rng.uniform(-W, W, n)
    gates = []
    for _ in range(layers):
        for q in range(n):
            gates.append(g("RZ", [q], [h[q] * dt]))
        for q in range(n - 1):
            gates += [g("Hadamard", [q]), g("Hadamard", [q + 1]), g("CNOT", [q, q + 1]),
                      g("RZ", [q + 1], [J * dt]), g("CNOT", [q, q + 1]),
                      g("Hadamard", [q]), g("Hadamard", [q + 1])]
            gates += [g("CNOT", [q, q + 1]), g("RZ", [q + 1], [J * dt]), g("CNOT", [q, q + 1])]
    return gates, [expval(("PauliZ", [q])) for q in range(n)]


def build_cases():
    rng = np.random.default_rng(20240601)
    cases = [{"name": nm, "n": n, "gates": gt, "meas": ms} for nm, n, gt, ms in case_reference_tests()]
    gt, ms = case_all_gates(rng)
    cases.append({"name": "all_gates_n4", "n": 4, "gates": gt, "meas": ms})
    gt, ms = case_all_gates(rng, n=5, depth=2)
    cases.append({"name": "all_gates_n5", "n": 5, "gates": gt, "meas": ms})
    cases.append({"name": "trainable_subsets", "n": 3, "gates": [
        g("Rot", [0], [0.3, 1.1, -0.7], trainable=[0, 2]),
        g("RZ", [1], [0.9], trainable=[]),
        g("Hadamard", [2]),
        g("PhaseShift", [2], [0.4], trainable=[]),
        g("CRY", [2, 1], [0.8]),
        g("Rot", [1], [0.2, -0.5, 1.3]),
        g("CNOT", [1, 0]),
        g("RY", [0], [0.6])],
        "meas": [expval(("PauliZ", [0])), expval(("PauliX", [1])), expval(("PauliY", [2]))]})
    cases.append({"name": "inverse_fixed", "n": 3, "gates": [
        g("Hadamard", [0]), g("Hadamard", [1]), g("Hadamard", [2]),
        g("S", [0], inv=True), g("T", [1], inv=True), g("SX", [2], inv=True),
        g("CY", [2, 0]), g("Toffoli", [0, 2, 1]), g("CSWAP", [1, 0, 2]), g("SWAP", [2, 0]),
        g("RX", [1], [0.37])],
        "meas": [{"kind": "state"}]})
    gt, ms = case_hea()
    cases.append({"name": "hea8", "n": 8, "gates": gt, "meas": ms})
    gt, ms = case_vqc(10, 2)
    cases.append({"name": "vqc10", "n": 10, "gates": gt, "meas": ms})
    gt, ms = case_mbl(rng, 8, 2)
    cases.append({"name": "mbl8", "n": 8, "gates": gt, "meas": ms})
    cases.append({"name": "probs_multi", "n": 4, "gates": [
        g("Hadamard", [0]), g("RY", [1], [0.7]), g("CNOT", [0, 2]), g("CRX", [1, 3], [1.9]),
        g("RZ", [3], [0.2]), g("CZ", [3, 0])],
        "meas": [{"kind": "probs", "qubits": [2, 0]}, {"kind": "probs", "qubits": [1, 3]}]})
    cases.append({"name": "controlled_orders", "n": 4, "gates": [
        g("Hadamard", [0]), g("Hadamard", [1]), g("Hadamard", [2]), g("Hadamard", [3]),
        g("CRX", [3, 0], [0.5]), g("CRY", [0, 3], [1.5]), g("CRZ", [2, 1], [2.5]),
        g("ControlledPhaseShift", [1, 3], [0.75]), g("PhaseShift", [0], [1.25]),
        g("CRZ", [0, 2], [-0.5]), g("CNOT", [3, 1]), g("RX", [2], [0.1])],
        "meas": [expval(("PauliX", [0])), expval(("PauliY", [1])), expval(("PauliZ", [2])),
                 expval(("PauliX", [3]), ("PauliX", [0]))]})
    cases.append({"name": "single_qubit", "n": 1, "gates": [
        g("Hadamard", [0]), g("RZ", [0], [0.3]), g("RY", [0], [1.2]), g("T", [0])],
        "meas": [expval(("PauliX", [0])), expval(("PauliY", [0])), expval(("PauliZ", [0]))]})
    cases.append({"name": "state_n6", "n": 6, "gates": case_all_gates(rng, n=6, depth=1)[0],
                  "meas": [{"kind": "state"}]})
    v = rng.normal(size=8) + 1j * rng.normal(size=8)
    v = v / np.linalg.norm(v)
    cases.append({"name": "init_state_n3", "n": 3, "init_state": [[float(x.real), float(x.imag)] for x in v],
                  "gates": [g("RX", [0], [0.4]), g("CNOT", [0, 2]), g("RY", [1], [1.1])],
                  "meas": [expval(("PauliZ", [0])), expval(("PauliX", [2]))]})
    for c in cases:
        c.setdefault("init_state", None)
        # every trainable angle gets a seeded value drawn like the benchmark configs
        for gg in c["gates"]:
            if c["name"].startswith(("hea", "vqc")):
                gg["params"] = [float(rng.uniform(0, 2 * np.pi)) for _ in gg["params"]]
    return cases


# --------------------------------------------------------------------------- running

def record(case, rdtype, param_shape=()):
    """Record ``case`` with the reference circuit API (refshim.record_circuit)."""
    return refshim.record_circuit(qai, case, rdtype, param_shape)


def flat_trainable(case):
    vals = []
    for gg in case["gates"]:
        vals += [gg["params"][i] for i in gg["trainable"]]
    return vals


def to_list(t):
    t = t.detach()
    if t.is_complex():
        return [[float(x.real), float(x.imag)] for x in t.reshape(-1)]
    return [float(x) for x in t.reshape(-1)]


def run_case(case, rng):
    out = {}
    for tag, cdt, rdt in (("c64", torch.complex64, torch.float32), ("c128", torch.complex128, torch.float64)):
        pb.tcomplex = cdt
        circ = record(case, rdt)
        cc = circ.compilecircuit(backend="pytorch")
        p = torch.tensor(flat_trainable(case), dtype=rdt, requires_grad=True)
        res = cc(p)
        out[f"out_{tag}"] = to_list(res)
        out["shape"] = list(res.shape)
        if p.numel() > 0:
            dy = case["_dy"]
            dyt = torch.tensor(dy, dtype=rdt).reshape(res.shape)
            loss = (res * dyt).real.sum() if res.is_complex() else (res * dyt).sum()
            loss.backward()
            out[f"grad_backprop_{tag}"] = to_list(p.grad)
    pb.tcomplex = torch.complex64
    if flat_trainable(case) and all(m["kind"] == "expval" for m in case["meas"]):
        circ = record(case, torch.float32)
        cc = circ.compilecircuit(backend="pytorch", diff_method="param_shift")
        p = torch.tensor(flat_trainable(case), dtype=torch.float32, requires_grad=True)
        res = cc(p)
        res.backward(torch.tensor(case["_dy"], dtype=torch.float32).reshape(res.shape))
        out["grad_paramshift_c64"] = to_list(p.grad)
    return out


def main():
    torch.manual_seed(0)
    rng = np.random.default_rng(7)
    cases = build_cases()
    result = []
    for c in cases:
        pb.tcomplex = torch.complex64
        shape = list(record(c, torch.float32).compilecircuit(backend="pytorch")(
            torch.tensor(flat_trainable(c), dtype=torch.float32)).shape)
        c["_dy"] = [float(x) for x in rng.normal(size=int(np.prod(shape)))]
        rec = run_case(c, rng)
        entry = {k: v for k, v in c.items() if not k.startswith("_")}
        entry["params"] = flat_trainable(c)
        entry["dy"] = c["_dy"]
        entry.update(rec)
        result.append(entry)
        print(f"{c['name']:22s} n={c['n']:2d} gates={len(c['gates']):4d} P={len(entry['params']):4d} out={rec['shape']}")
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference": "jd-opensource/TeD-Q",
                   "torch": torch.__version__, "cases": result}, f)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


# --------------------------------------------------------------------------- extended fixtures

class OEGreedy:
    """Stands in for the external ``JDOptTN`` path optimiser that the
    reference's ``use_jdopttn`` branch constructs and calls
    (compiled_circuit.py:388-393, pytorch_backend.py:339): the same
    constructor and ``contract(arrays, backend=...)``, with opt_einsum's greedy
    path (the default optimiser of the reference's OEWrapper)."""

    def __init__(self, inputs, size_dict, output=None, **kwargs):
        import opt_einsum
        self.eq = ",".join("".join(ix) for ix in inputs) + "->" + "".join(output or [])
        shapes = [tuple(size_dict[i] for i in ix) for ix in inputs]
        self.expr = opt_einsum.contract_expression(self.eq, *shapes, optimize="greedy")

    def contract(self, arrays, backend="torch", **kwargs):
        return self.expr(*arrays, backend=backend)


def lattice_case(rows, cols, layers, rng):
    gates = []
    for layer in range(layers):
        for q in range(rows * cols):
            gates.append(g("Rot", [q], [float(rng.uniform(0, 2 * np.pi)), float(np.arccos(rng.uniform(-1, 1))),
                                        float(rng.uniform(0, 2 * np.pi))]))
        par = (layer // 2) % 2
        if layer % 2 == 0:
            bonds = [(r * cols + c, r * cols + c + 1) for r in range(rows) for c in range(cols - 1) if c % 2 == par]
        else:
            bonds = [(r * cols + c, (r + 1) * cols + c) for r in range(rows - 1) for c in range(cols) if r % 2 == par]
        for a, b in bonds:
            gates.append(g("CZ", [a, b]))
    return gates


def random_case(rng, n, depth):
    gates = []
    for _ in range(depth):
        for q in range(n):
            gates.append(g(ROT1[int(rng.integers(3))], [q], [float(rng.uniform(0, 2 * np.pi))]))
        for q in range(int(rng.integers(2)), n - 1, 2):
            gates.append(g(["CNOT", "CZ"][int(rng.integers(2))], [q, q + 1]))
        gates.append(g("CRY", [int(rng.integers(n - 1)) + 1, 0], [float(rng.uniform(0, 2 * np.pi))]))
        gates.append(g("Hadamard", [int(rng.integers(n))]))
    return gates


def tn_cases(rng):
    """Circuits for the reference's tensor-network mode."""
    cases = []
    cases.append({"name": "tn_random_n5_expval", "n": 5, "gates": random_case(rng, 5, 3),
                  "meas": [expval(("PauliZ", [2])), expval(("PauliX", [0]), ("PauliY", [4])),
                           expval(("PauliZ", [1]), ("PauliZ", [3]))]})
    cases.append({"name": "tn_lattice_3x3_4layers", "n": 9, "gates": lattice_case(3, 3, 4, rng),
                  "meas": [expval(("PauliZ", [4]))]})
    cases.append({"name": "tn_random_n4_probs", "n": 4, "gates": random_case(rng, 4, 2),
                  "meas": [{"kind": "probs", "qubits": [2, 0]}, {"kind": "probs", "qubits": [1, 3]}]})
    cases.append({"name": "tn_random_n4_state", "n": 4, "gates": random_case(rng, 4, 2),
                  "meas": [{"kind": "state"}]})
    for c in cases:
        c["init_state"] = None
    return cases


def run_tn_case(case):
    out = {}
    for tag, cdt, rdt in (("c64", torch.complex64, torch.float32), ("c128", torch.complex128, torch.float64)):
        pb.tcomplex = cdt
        cc = record(case, rdt).compilecircuit(backend="pytorch", use_jdopttn=OEGreedy, tn_simplify=False)
        res = cc(torch.tensor(flat_trainable(case), dtype=rdt))
        out[f"out_{tag}"] = to_list(res)
        out["shape"] = list(res.shape)
    pb.tcomplex = torch.complex64
    return out


def after_state_case(rng):
    # a closing RY layer leaves every outcome of the measured qubits possible
    gates = random_case(rng, 4, 2) + [g("RY", [q], [float(rng.uniform(0.3, 2.8))]) for q in range(4)]
    return {"name": "after_state_n4", "n": 4, "init_state": None, "gates": gates,
            "meas": [{"kind": "probs", "qubits": [1, 2], "after_state": True}]}


def run_after_state(case):
    out = {}
    pb.tcomplex = torch.complex128
    cc = record(case, torch.float64).compilecircuit(backend="pytorch")
    res = cc(torch.tensor(flat_trainable(case), dtype=torch.float64))
    out["out_c128"] = to_list(res)
    out["shape"] = list(res.shape)
    after = cc.states_after_measurement
    out["after_states_c128"] = {k: to_list(torch.stack([torch.as_tensor(x) for x in v]))
                                for k, v in after.items()}
    pb.tcomplex = torch.complex64
    return out


def qng_case(rng, name, n, layers, kinds=None):
    gates = []
    for layer in range(layers):
        for q in range(n):
            kind = ["RX", "RY", "RZ"][int(rng.integers(3))] if kinds is None else kinds[layer][q]
            gates.append(g(kind, [q], [float(rng.uniform(0, 2 * np.pi))]))
        for q in range(n - 1):
            gates.append(g("CNOT", [q, q + 1]))
    gates.append(g("PhaseShift", [1], [float(rng.uniform(0, 2 * np.pi))]))
    return {"name": name, "n": n, "init_state": None, "gates": gates, "meas": [expval(("PauliZ", [0]))]}


def run_metric_tensor(case, numarg):
    pb.tcomplex = torch.complex64
    # metric_tensor runs the first layer's circuit with no call parameters
    # (parameters[:0], circuit.py:303): its gates keep the recorded values,
    # which the reference's gate builders need as 1-element tensors
    circ = record(case, torch.float32, param_shape=(1,))
    params = [torch.tensor([v], dtype=torch.float32) for v in flat_trainable(case)]
    mt = circ.metric_tensor(circ.gen_circuits(numarg), *params)
    return {"metric_tensor": [[float(x) for x in row] for row in mt.detach().double()], "numarg": list(numarg)}


def main_ext():
    rng = np.random.default_rng(20241204)
    result = {"tn": [], "after_state": [], "metric_tensor": []}
    for c in tn_cases(rng):
        rec = run_tn_case(c)
        entry = dict(c)
        entry["params"] = flat_trainable(c)
        entry.update(rec)
        result["tn"].append(entry)
        print(f"{c['name']:26s} n={c['n']:2d} gates={len(c['gates']):4d} out={rec['shape']}")
    c = after_state_case(rng)
    entry = dict(c)
    entry["params"] = flat_trainable(c)
    entry.update(run_after_state(c))
    result["after_state"].append(entry)
    print(f"{c['name']:26s} after states {sorted(entry['after_states_c128'])}")
    # the subset leaves parameter 1 unselected, so its RY on qubit 1 stays in
    # layer 0 ahead of parameter 0's gate (see run_metric_tensor)
    for name, n, layers, numarg, kinds in (
            ("qng_n4_l3_all", 4, 3, None, None),
            ("qng_n3_l2_subset", 3, 2, [0, 2, 4, 5], [["RY", "RY", "RX"], ["RX", "RY", "RY"]])):
        c = qng_case(np.random.default_rng(len(name) * 7919), name, n, layers, kinds)
        P = len(flat_trainable(c))
        # the last parameter is PhaseShift's: its generator builds the
        # reference's broken Unitary (qubit.py:1295, 1719), so it stays out
        na = list(range(P - 1)) if numarg is None else numarg
        entry = dict(c)
        entry["params"] = flat_trainable(c)
        entry.update(run_metric_tensor(c, na))
        result["metric_tensor"].append(entry)
        print(f"{name:26s} P={P} metric {len(entry['metric_tensor'])}x{len(entry['metric_tensor'])}")
    with open(OUT_EXT, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference": "jd-opensource/TeD-Q",
                   "torch": torch.__version__, **result}, f)
    print("wrote", OUT_EXT, os.path.getsize(OUT_EXT), "bytes")


if __name__ == "__main__":
    main()
    main_ext()
