"""Registers ``backend="gb300"`` with an installed reference ``tedq``.

The reference dispatches on the backend string in ``Circuit.compilecircuit``
(tedq/QInterpreter/circuits/circuit.py:268-285) and raises ``ValueError`` for
unknown strings.  ``register_with_tedq`` wraps that method so ``"gb300"``
constructs ``GB300Backend(backend, circuit, **kwargs)`` and every other string
goes to the original method; the reference's files are not modified.
``GB300Backend`` reads the reference's circuit objects through the same
attributes the reference's own ``CompiledCircuit`` reads.
"""


def register_with_tedq(tedq_module=None):
    """Wrap ``tedq``'s ``Circuit.compilecircuit``; returns True when done."""
    if tedq_module is None:
        try:
            import tedq as tedq_module  # noqa: F401
        except ImportError:
            return False
    from tedq.QInterpreter.circuits import circuit as circ_mod

    Circuit = circ_mod.Circuit
    if getattr(Circuit.compilecircuit, "_gb300_wrapped", False):
        return True
    original = Circuit.compilecircuit

    def compilecircuit(self, backend=None, **kwargs):
        if backend == "gb300":
            from .backend import GB300Backend
            return GB300Backend(backend, self, **kwargs)
        return original(self, backend, **kwargs)

    compilecircuit._gb300_wrapped = True
    compilecircuit.__doc__ = original.__doc__
    Circuit.compilecircuit = compilecircuit
    return True
