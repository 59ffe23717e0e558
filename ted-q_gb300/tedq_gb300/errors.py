"""Exception types of the reference (tedq/quantum_error.py:1-8)."""


class QuantumCircuitError(Exception):
    """The quantum circuit is malformed."""


class QuantumValueError(Exception):
    """A value is not available or not allowed."""


class QuantumStorageError(Exception):
    """The recording holds something that is not an operator or measurement."""


class BackendError(RuntimeError):
    """The native GB300 library reported an error."""
