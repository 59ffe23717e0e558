"""``Circuit``: records a user quantum function and compiles it.

Mirrors tedq/QInterpreter/circuits/circuit.py ``Circuit`` (:38-316): the
constructor runs ``func(*params)`` inside a recording, splits the recording
into state preparation, gates and measurements, and ``compilecircuit`` turns
it into an executable backend.  Here ``backend="gb300"`` selects the GB300
execution backend (``backend.GB300Backend``).
"""

import numpy as np

from . import _recording
from .errors import QuantumCircuitError, QuantumStorageError
from .measurement import QuantumMeasurement
from .operators import GateBase


def generate_parameters(parameter_shapes):
    """Random parameters for ``parameter_shapes`` (circuit.py:407-417)."""
    return tuple((np.random.rand(*shape) + 0.01) * np.e / 1.77 for shape in parameter_shapes)


class Circuit:
    def __init__(self, func, num_qubits, *params, **kwargs):
        if isinstance(func, dict):
            self._func = None
            self._operators = list(func["operators"])
            self._measurements = list(func["measurements"])
            self._init_state = func.get("init_state")
            self._num_qubits = num_qubits
        else:
            if not num_qubits:
                raise ValueError("Error in Circuit class, num_qubits cannot be None!")
            self._func = func
            self._num_qubits = num_qubits
            shapes = kwargs.get("parameter_shapes")
            if shapes:
                params = generate_parameters(shapes)
            with _recording.CircuitStorage() as store:
                func(*params)
            ctx = store.storage_context
            self._init_state = ctx[0] if ctx and getattr(ctx[0], "is_preparation", False) else None
            self._operators = [o for o in ctx if isinstance(o, GateBase)]
            self._measurements = [o for o in ctx if isinstance(o, QuantumMeasurement)]
            if len(self._operators) + len(self._measurements) + bool(self._init_state) != len(ctx):
                raise QuantumStorageError("Error in Circuit class, unknown content in the storage_context!")
        if not self._measurements:
            raise QuantumCircuitError("No measurement! please specify a quantum measurement!")
        top = self.maximum_qubit_num()
        if top + 1 > self._num_qubits:
            raise ValueError(f"Input number of qubits is not large enough! Maximum qubit number of operators "
                             f"is {top + 1}")

    def maximum_qubit_num(self):
        top = 0
        for op in self._operators:
            top = max(top, max(op.qubits))
        for m in self._measurements:
            if m.qubits is not None and len(m.qubits):
                top = max(top, max(m.qubits))
            if m.obs is not None:
                for ob in (m.obs if isinstance(m.obs, list) else [m.obs]):
                    top = max(top, max(ob.qubits))
        return top

    @property
    def operators(self):
        return self._operators

    @property
    def num_qubits(self):
        return self._num_qubits

    @property
    def measurements(self):
        return self._measurements

    @property
    def init_state(self):
        return self._init_state

    # ------------------------------------------------ quantum natural gradient
    def cycabc(self, numarg):
        """Layering for the metric tensor (circuit.py:101-164)."""
        from .qng import layer_blocks
        return layer_blocks(self, numarg)

    def gen_circuits(self, numarg, **kwargs):
        """Per-layer circuits of the metric tensor (circuit.py:166-203), compiled
        for the GB300 backend; returns the ``MetricTensor`` that
        ``metric_tensor`` evaluates (the reference returns a list of circuits
        compiled again on every call)."""
        from .qng import MetricTensor
        return MetricTensor(self, numarg, **kwargs)

    def metric_tensor(self, circuits_list, *parameters):
        """Block-diagonal metric tensor (circuit.py:297-316) for the circuit's
        flat parameters."""
        return circuits_list(*parameters)

    def compilecircuit(self, backend=None, **kwargs):
        """Compile for ``backend``; ``"gb300"`` is the GB300 backend."""
        if backend == "gb300":
            from .backend import GB300Backend
            return GB300Backend(backend, self, **kwargs)
        if backend == "gb300_QUDIO":
            from .backend import GB300QUDIO
            return GB300QUDIO(backend, self, **kwargs)
        raise ValueError(f"{backend}: unknown backend input")

    def __str__(self):
        lines = ["# operators"]
        lines += [f"qai.{g.name}(qubits={g.qubits})" for g in self.operators]
        lines += ["", "", "# measurements"]
        for m in self.measurements:
            if m.obs is not None and not isinstance(m.obs, list):
                lines.append(f"qai.measurement.expval(qai.{m.obs.name}(qubits={m.obs.qubits}))")
            else:
                lines.append(f"qai.measurement.{m.return_type.value}(...)")
        return "\n".join(lines) + "\n"

    @classmethod
    def from_spec(cls, spec):
        """Record a circuit from a neutral description (the dict format of the
        golden fixtures: ``n``, ``gates``, ``meas``, ``init_state``)."""
        from . import operators as O
        from .measurement import expval, probs, state

        def circuit_def():
            if spec.get("init_state") is not None:
                a = np.asarray(spec["init_state"], dtype=np.float64)
                O.IintStateVector(a[:, 0] + 1j * a[:, 1], qubits=[])
            for g in spec["gates"]:
                if g["name"] == "Unitary":
                    a = np.asarray(g["matrix"], dtype=np.float64)
                    op = O.Unitary(a[:, 0] + 1j * a[:, 1], qubits=g["qubits"], trainable_params=[])
                else:
                    op = getattr(O, g["name"])(*g["params"], qubits=g["qubits"], trainable_params=g["trainable"])
                if g.get("inv"):
                    op.inverse()
            for m in spec["meas"]:
                if m["kind"] == "expval":
                    obs = [getattr(O, o["name"])(qubits=o["qubits"]) for o in m["obs"]]
                    expval(obs if m.get("list", len(obs) > 1) else obs[0])
                elif m["kind"] == "probs":
                    probs(qubits=m["qubits"], after_state=bool(m.get("after_state", False)))
                else:
                    state()
        return cls(circuit_def, spec["n"])
