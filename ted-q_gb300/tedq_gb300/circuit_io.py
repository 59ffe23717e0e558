"""Circuit ingestion from qsim-style text files.

Mirrors tedq/QInterpreter/circuits/circuit_io.py (:24-142): the first line is
the number of qubits, every further line ``<moment> <gate> <qubits...>
<params...>``; ``FromQasmFile(path)`` parses once and, when called inside a
circuit definition, records the gates.  Gate names: x, y, z, h, s, x_1_2
(SX), cnot, rx, ry, rz as in the reference, plus t and cz.
"""

from . import operators as O

_GATES = {
    "x": (O.PauliX, 1, 0), "y": (O.PauliY, 1, 0), "z": (O.PauliZ, 1, 0), "h": (O.Hadamard, 1, 0),
    "s": (O.S, 1, 0), "t": (O.T, 1, 0), "x_1_2": (O.SX, 1, 0), "cnot": (O.CNOT, 2, 0), "cz": (O.CZ, 2, 0),
    "rx": (O.RX, 1, 1), "ry": (O.RY, 1, 1), "rz": (O.RZ, 1, 1),
}


def _number(tok):
    for conv in (int, float):
        try:
            return conv(tok)
        except ValueError:
            pass
    return tok


def parse_qasm(lines):
    """``{'n_qubits': int, 'gates': [tuple]}`` from an iterable of lines."""
    lines = [ln.rstrip("\n") for ln in lines]
    if not lines:
        raise ValueError("empty circuit file")
    n_qubits = int(lines[0])
    gates = [tuple(_number(t) for t in ln.strip().split()) for ln in lines[1:] if ln.strip()]
    return {"n_qubits": n_qubits, "gates": gates}


def parse_qasm_file(fname, encoding="utf-8"):
    with open(fname, "r", encoding=encoding) as fh:
        return parse_qasm(fh)


def convert_to_tedq_format(gate):
    """``(gate class, qubits, parameters)`` of one parsed line."""
    try:
        cls, wires, n_pars = _GATES[gate[1]]
    except KeyError as error:
        raise ValueError("This gate from qasm file is not supported yet!!!") from error
    qubits = list(gate[2:2 + wires])
    pars = list(gate[2 + wires:2 + wires + n_pars])
    if len(qubits) != wires or len(pars) != n_pars:
        raise ValueError(f"malformed gate line: {gate}")
    return cls, qubits, pars


class FromQasmFile:
    """Reads a circuit file; calling the object records its gates."""

    def __init__(self, fname):
        info = parse_qasm_file(fname)
        self._n_qubits = info["n_qubits"]
        self._operands = [convert_to_tedq_format(g) for g in info["gates"]]
        for _, qubits, _ in self._operands:
            if max(qubits) >= self._n_qubits:
                raise ValueError("gate qubit index out of range of the file's qubit count")

    def __call__(self):
        for cls, qubits, pars in self._operands:
            cls(*pars, qubits=qubits)

    @property
    def n_qubits(self):
        return self._n_qubits
