"""Time the reference against the oracle's restatement of it (the "port"
that ``bench.py --impl reference`` runs on machines without the reference).

    python tests/golden/calibrate_port.py [--qubits 20] [--layers 10] [--circuits 2] [--threads N]

Both run the benchmark's circuit (RX, RY, RZ on every qubit and a CNOT ladder
per layer; <Z_i> on every qubit and <Z_0 Z_1>) value + gradient by back_prop
in complex64 on the same host threads, the reference through its own circuit
API and ``PyTorchBackend`` (imported unmodified, ``refshim``), the port
through ``oracle.value_and_grad``, alternating circuit by circuit with the
same parameters.  Prints one JSON line with seconds per circuit of each and
their ratio.
"""

import argparse
import json
import os
import platform
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import refshim  # noqa: E402


def vqc_gates(n, layers, rng):
    gates = []
    for _ in range(layers):
        for q in range(n):
            for name in ("RX", "RY", "RZ"):
                gates.append((name, [q], float(rng.uniform(0, 2 * np.pi))))
        for q in range(n - 1):
            gates.append(("CNOT", [q, q + 1], None))
    return gates


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, default=20)
    ap.add_argument("--layers", type=int, default=10)
    ap.add_argument("--circuits", type=int, default=2)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--reference", default=refshim.DEFAULT_PATH)
    a = ap.parse_args()
    if a.threads:
        torch.set_num_threads(a.threads)
    tq = refshim.import_reference(a.reference)
    import oracle

    n = a.qubits
    gates = vqc_gates(n, a.layers, np.random.default_rng(0))

    def circuit_def(*p):
        for name, qs, th in gates:
            if th is None:
                getattr(tq, name)(qubits=qs)
            else:
                getattr(tq, name)(torch.tensor(th), qubits=qs)
        return [tq.expval(tq.PauliZ(qubits=[q])) for q in range(n)] + \
               [tq.expval([tq.PauliZ(qubits=[0]), tq.PauliZ(qubits=[1])])]

    ref = tq.Circuit(circuit_def, n).compilecircuit(backend="pytorch")
    spec = {"n": n, "init_state": None,
            "gates": [{"name": name, "qubits": qs, "params": [] if th is None else [th],
                       "trainable": [] if th is None else [0]} for name, qs, th in gates],
            "meas": [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n)]
            + [{"kind": "expval", "list": True, "obs": [{"name": "PauliZ", "qubits": [0]},
                                                        {"name": "PauliZ", "qubits": [1]}]}]}
    P = sum(1 for g in gates if g[2] is not None)
    gen = torch.Generator().manual_seed(1)
    dy = np.ones(n + 1)
    t_ref, t_port, err = [], [], 0.0
    for i in range(a.circuits + 1):  # the first circuit of each is a warm-up
        p = torch.rand(P, generator=gen) * 2 * np.pi
        t0 = time.perf_counter()
        pr = p.clone().requires_grad_(True)
        out = ref(pr)
        out.sum().backward()
        t1 = time.perf_counter()
        v, gr = oracle.value_and_grad(spec, p.clone(), dy, torch.complex64)
        t2 = time.perf_counter()
        if i:
            t_ref.append(t1 - t0)
            t_port.append(t2 - t1)
        err = max(err, float((out.detach().double().reshape(-1) - torch.as_tensor(v).double().reshape(-1)).abs().max()),
                  float((pr.grad.double() - torch.as_tensor(gr).double()).abs().max()))
    r, q = float(np.mean(t_ref)), float(np.mean(t_port))
    print(json.dumps({"circuit": f"vqc{n}q_{a.layers}layers", "circuits": a.circuits,
                      "threads": torch.get_num_threads(), "cpu_count": os.cpu_count(), "cpu_model": cpu_model(),
                      "torch": torch.__version__, "reference_s_per_circuit": r, "port_s_per_circuit": q,
                      "port_over_reference": q / r, "max_abs_diff": err}))


if __name__ == "__main__":
    main()
