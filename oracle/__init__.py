"""CPU oracle for TeD-Q's compiled-circuit state-vector path.

TEST INFRASTRUCTURE ONLY.  This package restates, on the host CPU with torch,
what the reference's ``PyTorchBackend`` does (tedq/backends/pytorch_backend.py,
tedq/backends/compiled_circuit.py, tedq/QInterpreter/operators/qubit.py).
It is the checker for the CUDA path: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` may import it.  The product package never imports it and has no
CPU fallback.

Parity pinning: the restatement is checked against golden vectors produced by
the reference itself (``tests/golden/make_golden.py`` imports the reference
and records its outputs) and against the literal known-answer values in the
reference's own tests (test/test_pytorch_backend.py:386-584).
"""

from .sv_oracle import (  # noqa: F401
    GATE_ARITY,
    GATE_NPARAMS,
    spec_from_circuit,
    gate_matrix_fixed,
    bind_parameters,
    run,
    param_shift_jacobian,
    value_and_grad,
    pauli_expval_from_state,
)
