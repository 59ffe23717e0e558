"""Recording context for circuit construction.

Mirrors the reference's global deque of active storages
(tedq/_set_global_variables.py:7, tedq/QInterpreter/circuits/storage_base.py
``StorageBase``/``CircuitStorage`` :28-162): operators and measurements
append themselves to the innermost active ``CircuitStorage``.
"""

from collections import deque

_active = deque()


class CircuitStorage:
    """Context manager collecting everything recorded inside it."""

    def __init__(self):
        self.storage_context = []

    def __enter__(self):
        _active.append(self)
        return self

    def __exit__(self, exc_type, exc, tb):
        _active.pop()

    def _append(self, obj):
        self.storage_context.append(obj)

    def _remove(self, obj):
        self.storage_context.remove(obj)


def recording():
    return bool(_active)


def active():
    return _active[-1] if _active else None


def append(obj):
    """Append to the active recording; ValueError outside one (ops_abc.py:62-75)."""
    if not _active:
        raise ValueError("There's no global_deque for storing information!")
    _active[-1]._append(obj)
