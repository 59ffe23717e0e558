"""tedq_gb300 -- GB300 (sm_103a) execution backend for TeD-Q compiled circuits.

The circuit-recording API mirrors the reference's ``tedq`` package
(``Circuit``, the gate/observable classes, ``expval``/``probs``/``state``) so
circuits written for TeD-Q run unchanged with ``import tedq_gb300 as qai`` and
``circuit.compilecircuit(backend="gb300")``.  ``register_with_tedq()`` adds the
same backend string to an installed reference ``tedq``.
"""

import os as _os

# Hardware work queues per CUDA context (read when the context is created,
# i.e. effective when this package is imported before the first CUDA call).
# The driver's default of 8 makes streams share queues, and a kernel then
# waits in order behind another stream's kernels: the serving loop's
# high-priority small-circuit streams would queue behind large circuits.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from .circuit import Circuit, generate_parameters  # noqa: F401,E402
from .errors import BackendError, QuantumCircuitError, QuantumStorageError, QuantumValueError  # noqa: F401
from .measurement import (Expectation, MeasurementReturnTypes, Probability, QuantumMeasurement,  # noqa: F401
                          State, expval, probs, sample, state, var)
from .operators import (CNOT, CRX, CRY, CRZ, CSWAP, CY, CZ, RX, RY, RZ, SWAP, SX, ControlledPhaseShift,  # noqa: F401
                        GateBase, Hadamard, I, IintStateVector, ObservableBase, OperatorBase, PauliX, PauliY,
                        PauliZ, PhaseShift, Rot, S, T, Toffoli, Unitary)
from .backend import GB300QUDIO, GB300Backend, GB300Execute, GB300ParamShift, GB300TnExecute  # noqa: F401
from .circuit_io import FromQasmFile  # noqa: F401
from .qng import QNG, MetricTensor  # noqa: F401
from .reference_bridge import register_with_tedq  # noqa: F401

__version__ = "0.1.0"
