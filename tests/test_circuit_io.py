"""qsim-style text ingestion (circuit_io.py:24-142 of the reference): parsing,
the reference's own test case, and execution against the oracle."""

import numpy as np
import pytest
import torch

import oracle

qai = pytest.importorskip("tedq_gb300")


def _write(tmp_path, text):
    p = tmp_path / "c.qsim"
    p.write_text(text)
    return str(p)


def test_reads_three_qubit_file(tmp_path):
    # the layout of the reference's test/test.qsim (test_circuit.py:248-263)
    q = qai.FromQasmFile(_write(tmp_path, "3\n0 x 0\n0 y 1\n0 x 2"))
    assert q.n_qubits == 3

    def circuit_def():
        q()
        return qai.expval(qai.PauliZ(qubits=[0]))

    circ = qai.Circuit(circuit_def, q.n_qubits)
    assert circ.operators[2].qubits == [2]
    assert [op.name for op in circ.operators] == ["PauliX", "PauliY", "PauliX"]


def test_parameterised_lines_and_errors(tmp_path):
    q = qai.FromQasmFile(_write(tmp_path, "2\n0 h 0\n1 cnot 0 1\n2 rx 1 0.5\n2 rz 0 -1.25\n3 x_1_2 1\n"))

    def circuit_def():
        q()
        return qai.expval(qai.PauliZ(qubits=[1]))

    circ = qai.Circuit(circuit_def, q.n_qubits)
    names = [op.name for op in circ.operators]
    assert names == ["Hadamard", "CNOT", "RX", "RZ", "SX"]
    assert float(circ.operators[2].parameters[0]) == 0.5
    with pytest.raises(ValueError):
        qai.FromQasmFile(_write(tmp_path, "2\n0 fsim 0 1 0.1 0.2\n"))
    with pytest.raises(ValueError):
        qai.FromQasmFile(_write(tmp_path, "2\n0 x 3\n"))


@pytest.mark.gpu
def test_file_circuit_runs_on_gpu(tmp_path):
    rng = np.random.default_rng(0)
    lines = ["6"]
    for m in range(20):
        kind = rng.choice(["h", "x_1_2", "cnot", "rx", "ry", "rz", "t", "cz"])
        if kind in ("cnot", "cz"):
            a, b = rng.choice(6, 2, replace=False)
            lines.append(f"{m} {kind} {a} {b}")
        elif kind in ("rx", "ry", "rz"):
            lines.append(f"{m} {kind} {rng.integers(6)} {rng.uniform(0, 6.28):.6f}")
        else:
            lines.append(f"{m} {kind} {rng.integers(6)}")
    q = qai.FromQasmFile(_write(tmp_path, "\n".join(lines)))

    def circuit_def():
        q()
        return [qai.expval(qai.PauliZ(qubits=[i])) for i in range(6)]

    circ = qai.Circuit(circuit_def, q.n_qubits)
    flat = [float(op.parameters[t]) for op in circ.operators for t in op.trainable_params]
    cc = circ.compilecircuit(backend="gb300", precision="c128", requires_grad=False)
    out = cc(torch.tensor(flat, dtype=torch.float64)) if flat else cc()
    want = oracle.run(oracle.spec_from_circuit(circ), torch.tensor(flat, dtype=torch.float64),
                      torch.complex128).numpy()
    np.testing.assert_allclose(out.cpu().numpy(), want, atol=1e-12)
