"""Measurements: ``expval``, ``probs``, ``state``, ``var``, ``sample``.

Mirrors tedq/QInterpreter/operators/measurement.py (``QuantumMeasurement``
:29-103, ``expval`` :106-155, ``probs`` :174-207, ``state`` :210-237, return
types :240-266).  ``expval`` replaces the just-recorded observable(s) in the
active recording by the measurement, exactly as the reference does.
"""

from enum import Enum

from . import _recording
from .errors import QuantumCircuitError, QuantumValueError
from .operators import ObservableBase


class MeasurementReturnTypes(Enum):
    Sample = "sample"
    Variance = "var"
    Expectation = "expval"
    Probability = "probs"
    State = "state"

    def __repr__(self):
        return str(self.value)


Sample = MeasurementReturnTypes.Sample
Variance = MeasurementReturnTypes.Variance
Expectation = MeasurementReturnTypes.Expectation
Probability = MeasurementReturnTypes.Probability
State = MeasurementReturnTypes.State


class QuantumMeasurement:
    def __init__(self, return_type, obs=None, qubits=None, do_queue=True, after_state=False):
        self.return_type = return_type
        self.obs = obs
        self.do_queue = do_queue
        self.after_state = after_state
        if qubits is not None and obs is not None:
            raise ValueError("If an observable is provied, the qubit(s) can not be specified!")
        self.qubits = qubits
        if self.do_queue:
            self._queue()

    def _queue(self):
        store = _recording.active()
        if store is None:
            raise QuantumCircuitError("No active warehouse: measurements must be recorded inside a Circuit")
        if self.obs is not None:
            obs = self.obs if isinstance(self.obs, list) else [self.obs]
            for ob in reversed(obs):
                last = store.storage_context[-1] if store.storage_context else None
                if last is not None and getattr(last, "instance_id", None) == ob.instance_id:
                    store._remove(ob)
                else:
                    raise ValueError("Last content operator should be the same as 'obs'!")
        store._append(self)


def expval(observable, do_queue=True):
    """Expectation value of an observable or of a tensor product (list)."""
    for ob in (observable if isinstance(observable, list) else [observable]):
        if not isinstance(ob, ObservableBase):
            raise QuantumValueError(f"{ob.name} is not a subclass of ObservableBase: cannot be used with expval")
    return QuantumMeasurement(Expectation, obs=observable, do_queue=do_queue)


def _check_obs(observable):
    for ob in (observable if isinstance(observable, list) else [observable]):
        if not isinstance(ob, ObservableBase):
            raise QuantumValueError(f"{ob.name} is not a subclass of ObservableBase: cannot be used here")


def var(observable, do_queue=True):
    """Variance <O^2> - <O>^2 of an observable or tensor product (declared but
    not implemented by the reference, measurement.py:158-163)."""
    _check_obs(observable)
    return QuantumMeasurement(Variance, obs=observable, do_queue=do_queue)


def sample(observable, num_shots, do_queue=True):
    """``num_shots`` eigenvalue samples of an observable or tensor product,
    drawn from the state's distribution in the observable's eigenbasis
    (declared but not implemented by the reference, measurement.py:166-171)."""
    _check_obs(observable)
    if int(num_shots) < 1:
        raise QuantumValueError("num_shots must be positive")
    m = QuantumMeasurement(Sample, obs=observable, do_queue=do_queue)
    m.num_shots = int(num_shots)
    return m


def probs(qubits=None, do_queue=True, after_state=False):
    """Computational-basis probabilities of ``qubits`` (all qubits if None)."""
    return QuantumMeasurement(Probability, qubits=qubits, do_queue=do_queue, after_state=after_state)


def state(do_queue=True):
    """The final state vector."""
    return QuantumMeasurement(State, do_queue=do_queue)
