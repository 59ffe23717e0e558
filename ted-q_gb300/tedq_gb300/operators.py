"""Gate, observable and state-preparation classes of the circuit-recording API.

Mirrors the reference's operator model (tedq/QInterpreter/operators/ops_abc.py
``OperatorBase`` :28-220, ``GateBase`` :227-340, ``ObservableBase`` :343-380;
qubit.py gate classes :44-1786; prepared_state.py ``IintStateVector`` :29-57)
so that circuits written for TeD-Q record unchanged: same class names,
constructor signature ``Gate(*params, qubits=[...], do_queue=True,
trainable_params=[...])``, the same ``matrix`` convention (qubits[0] is the
most significant factor) and the same errors.

Operators record themselves into the active circuit recording (see
``circuit.py``); constructing one with ``do_queue=True`` outside a recording is
a ``ValueError`` as in the reference (ops_abc.py:62-75).
"""

import cmath
import itertools
import math

import numpy as np

from . import _recording

_INV_SQRT2 = 1.0 / math.sqrt(2.0)

# Parameter-shift recipes [(multiplier, scale, shift), ...]:
# default two-term rule (ops_abc.py:261-280) and the four-term rule of the
# controlled rotations (qubit.py:32-42).
_SHIFT = np.pi / 2.0
DEFAULT_SHIFT_RECIPE = [[0.5 / np.sin(_SHIFT), 1.0, _SHIFT], [-0.5 / np.sin(_SHIFT), 1.0, -_SHIFT]]
_M1 = _INV_SQRT2 * (np.sqrt(2) + 1) / 4
_M2 = _INV_SQRT2 * (np.sqrt(2) - 1) / 4
CONTROL_SHIFT_RECIPE = [[_M1, 1.0, np.pi / 2], [-_M1, 1.0, -np.pi / 2],
                        [-_M2, 1.0, 3 * np.pi / 2], [_M2, 1.0, -3 * np.pi / 2]]


def _f(x):
    """Plain float of a recorded parameter (number, 0-d or 1-element tensor/array)."""
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return float(x.detach().reshape(-1)[0])
    except ImportError:  # pragma: no cover
        pass
    return float(np.asarray(x).reshape(-1)[0])


class OperatorBase:
    """Common part of gates, observables and state preparations."""

    _count = itertools.count()
    _num_params = 0
    _num_qubits = 1

    def __init__(self, *params, qubits, do_queue=True, **kwargs):
        self._name = self.__class__.__name__
        if len(params) != self.num_params:
            raise ValueError(f"{self._name}: # of parameters is not matched! expected {self.num_params}"
                             f"parameters, but got {len(params)}.")
        qubits = list(qubits)
        if self.num_qubits is not None and len(qubits) != self.num_qubits:
            raise ValueError(f"{self._name}: # of qubits this operator applied on is not matched! expected "
                             f"{self.num_qubits} qubits, but got {len(qubits)}")
        self._instance_id = next(OperatorBase._count)
        self._do_queue = do_queue
        self._qubits = qubits
        self._params = list(params)
        self._trainable_params = list(kwargs.pop("trainable_params", list(range(self.num_params))))
        self._is_preparation = kwargs.pop("is_preparation", False)
        self._expected_index = kwargs.pop("expected_index", 0)
        if do_queue:
            _recording.append(self)
        self._matrix = self.get_matrix()

    def get_matrix(self):
        raise NotImplementedError

    @property
    def matrix(self):
        return self._matrix

    @property
    def eigvals(self):
        return np.linalg.eigvals(self.matrix)

    @property
    def num_params(self):
        return self._num_params

    @property
    def num_qubits(self):
        return self._num_qubits

    @property
    def name(self):
        return self._name

    @property
    def qubits(self):
        return self._qubits

    @property
    def parameters(self):
        return self._params

    @property
    def instance_id(self):
        return self._instance_id

    @property
    def trainable_params(self):
        return self._trainable_params

    @property
    def is_preparation(self):
        return self._is_preparation


class GateBase(OperatorBase):
    """A unitary gate (ops_abc.py:227-340)."""

    def __init__(self, *params, qubits, do_queue=True, **kwargs):
        self._inverse = False
        super().__init__(*params, qubits=qubits, do_queue=do_queue, **kwargs)

    @property
    def grad_style(self):
        return "param-shift" if self.num_params > 0 else None

    def get_parameter_shift(self):
        if self.grad_style == "param-shift":
            return DEFAULT_SHIFT_RECIPE
        raise ValueError(f"{self.name} : This quantum gate do not support parameter-shift method")

    @property
    def is_inverse(self):
        return self._inverse

    def inverse(self):
        """Turn this instance into its inverse: name gets ``.inv``, matrix is
        conjugate-transposed (ops_abc.py:293-325)."""
        if self._inverse:
            self._inverse = False
            self._name = self._name[:-4]
        else:
            self._inverse = True
            self._name = self._name + ".inv"
        self._matrix = self._matrix.conj().T
        return self

    def adjoint(self, do_queue=False):
        raise NotImplementedError


class ObservableBase(OperatorBase):
    """An observable usable in ``expval`` (ops_abc.py:343-380)."""

    return_type = None

    def diagonalizing_gates(self):
        raise NotImplementedError


class _Fixed1(GateBase):
    _num_params = 0
    _num_qubits = 1
    _M = None

    def get_matrix(self):
        return np.array(self._M, dtype=np.complex128)

    def adjoint(self, do_queue=False):
        return type(self)(qubits=self.qubits, do_queue=do_queue).inverse() if not self._self_adjoint \
            else type(self)(qubits=self.qubits, do_queue=do_queue)

    _self_adjoint = True


class Hadamard(ObservableBase, _Fixed1):
    _M = [[_INV_SQRT2, _INV_SQRT2], [_INV_SQRT2, -_INV_SQRT2]]

    def diagonalizing_gates(self, do_queue=False):
        return [RY(-np.pi / 4, qubits=self.qubits, do_queue=do_queue)]


class PauliX(ObservableBase, _Fixed1):
    _M = [[0, 1], [1, 0]]

    def diagonalizing_gates(self, do_queue=False):
        return [Hadamard(qubits=self.qubits, do_queue=do_queue)]


class PauliY(ObservableBase, _Fixed1):
    _M = [[0, -1j], [1j, 0]]

    def diagonalizing_gates(self, do_queue=False):
        return [PauliZ(qubits=self.qubits, do_queue=do_queue), S(qubits=self.qubits, do_queue=do_queue),
                Hadamard(qubits=self.qubits, do_queue=do_queue)]


class PauliZ(ObservableBase, _Fixed1):
    _M = [[1, 0], [0, -1]]

    def diagonalizing_gates(self, do_queue=False):
        return [I(qubits=self.qubits, do_queue=do_queue)]


class I(ObservableBase, _Fixed1):  # noqa: E742
    _M = [[1, 0], [0, 1]]

    def diagonalizing_gates(self, do_queue=False):
        return [I(qubits=self.qubits, do_queue=do_queue)]


class S(_Fixed1):
    _M = [[1, 0], [0, 1j]]
    _self_adjoint = False


class T(_Fixed1):
    _M = [[1, 0], [0, cmath.exp(1j * np.pi / 4)]]
    _self_adjoint = False


class SX(_Fixed1):
    _M = [[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]]
    _self_adjoint = False


class _FixedN(GateBase):
    _num_params = 0
    _M = None

    def get_matrix(self):
        return np.array(self._M, dtype=np.complex128)

    def adjoint(self, do_queue=False):
        return type(self)(qubits=self.qubits, do_queue=do_queue)


class CNOT(_FixedN):
    _num_qubits = 2
    _M = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]


class CZ(_FixedN):
    _num_qubits = 2
    _M = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, -1]]


class CY(_FixedN):
    _num_qubits = 2
    _M = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]]


class SWAP(_FixedN):
    _num_qubits = 2
    _M = [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]


class CSWAP(_FixedN):
    _num_qubits = 3
    _M = np.eye(8)[[0, 1, 2, 3, 4, 6, 5, 7]]


class Toffoli(_FixedN):
    _num_qubits = 3
    _M = np.eye(8)[[0, 1, 2, 3, 4, 5, 7, 6]]


class _Param(GateBase):
    _num_params = 1
    _num_qubits = 1

    def adjoint(self, do_queue=False):
        return type(self)(*[-p for p in self.parameters], qubits=self.qubits, do_queue=do_queue)


class RX(_Param):
    def get_matrix(self):
        th = _f(self._params[0])
        c, js = math.cos(th / 2), 1j * math.sin(-th / 2)
        return np.array([[c, js], [js, c]])

    @property
    def generator(self):
        return [-0.5, PauliX(qubits=self.qubits, do_queue=False)]


class RY(_Param):
    def get_matrix(self):
        th = _f(self._params[0])
        c, s = math.cos(th / 2), math.sin(th / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)

    @property
    def generator(self):
        return [-0.5, PauliY(qubits=self.qubits, do_queue=False)]


class RZ(_Param):
    def get_matrix(self):
        p = cmath.exp(-0.5j * _f(self._params[0]))
        return np.array([[p, 0], [0, p.conjugate()]])

    @property
    def generator(self):
        return [-0.5, PauliZ(qubits=self.qubits, do_queue=False)]


class Rot(GateBase):
    """Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi) (qubit.py:1137-1224)."""

    _num_params = 3
    _num_qubits = 1

    def get_matrix(self):
        phi, theta, omega = (_f(p) for p in self._params)
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return np.array([[cmath.exp(-0.5j * (phi + omega)) * c, -cmath.exp(0.5j * (phi - omega)) * s],
                         [cmath.exp(-0.5j * (phi - omega)) * s, cmath.exp(0.5j * (phi + omega)) * c]])

    @staticmethod
    def decomposition(phi, theta, omega, qubits, do_queue=False):
        return [RZ(phi, qubits=qubits, do_queue=do_queue), RY(theta, qubits=qubits, do_queue=do_queue),
                RZ(omega, qubits=qubits, do_queue=do_queue)]

    def adjoint(self, do_queue=False):
        phi, theta, omega = self.parameters
        return Rot(-omega, -theta, -phi, qubits=self.qubits, do_queue=do_queue)


class PhaseShift(_Param):
    def get_matrix(self):
        return np.array([[1, 0], [0, cmath.exp(1j * _f(self._params[0]))]])

    @property
    def generator(self):
        return [1, Unitary(np.array([[0, 0], [0, 1]], dtype=np.complex64), qubits=self.qubits, do_queue=False)]


class ControlledPhaseShift(_Param):
    _num_qubits = 2

    def get_matrix(self):
        return np.diag([1, 1, 1, cmath.exp(1j * _f(self._params[0]))])

    @property
    def generator(self):
        return [1, Unitary(np.diag([0, 0, 0, 1]).astype(np.complex64), qubits=self.qubits, do_queue=False)]


class _CRot(_Param):
    _num_qubits = 2

    def get_parameter_shift(self):
        if self.grad_style == "param-shift":
            return CONTROL_SHIFT_RECIPE
        raise ValueError(f"{self.name} : This quantum gate do not support parameter-shift method")


class CRX(_CRot):
    def get_matrix(self):
        th = _f(self._params[0])
        c, js = math.cos(th / 2), 1j * math.sin(-th / 2)
        return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, c, js], [0, 0, js, c]])

    @property
    def generator(self):
        g = np.zeros((4, 4), dtype=np.complex64)
        g[2:, 2:] = [[0, 1], [1, 0]]
        return [-0.5, Unitary(g, qubits=self.qubits, do_queue=False)]


class CRY(_CRot):
    def get_matrix(self):
        th = _f(self._params[0])
        c, s = math.cos(th / 2), math.sin(th / 2)
        return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, c, -s], [0, 0, s, c]], dtype=np.complex128)

    @property
    def generator(self):
        g = np.zeros((4, 4), dtype=np.complex64)
        g[2:, 2:] = [[0, -1j], [1j, 0]]
        return [-0.5, Unitary(g, qubits=self.qubits, do_queue=False)]


class CRZ(_CRot):
    def get_matrix(self):
        th = _f(self._params[0])
        return np.diag([1, 1, cmath.exp(-0.5j * th), cmath.exp(0.5j * th)])

    @property
    def generator(self):
        return [-0.5, Unitary(np.diag([0, 0, 1, -1]).astype(np.complex64), qubits=self.qubits, do_queue=False)]


class Unitary(GateBase, ObservableBase):
    """User-defined fixed matrix on ``len(qubits)`` qubits (qubit.py:1696-1786).

    The reference's constructor fails (it diagonalises an undefined name,
    qubit.py:1719); here the matrix is accepted as given."""

    _num_params = 0
    _num_qubits = None

    def __init__(self, matrix, qubits, do_queue=True, **kwargs):
        self._num_qubits = len(list(qubits))
        k = self._num_qubits
        self._user_defined_matrix = np.asarray(matrix, dtype=np.complex128).reshape(2 ** k, 2 ** k)
        super().__init__(qubits=qubits, do_queue=do_queue, **kwargs)
        vals, vecs = np.linalg.eig(self._user_defined_matrix)
        self._eigvals = vals
        self._diagonalizing_matrix = np.linalg.inv(vecs)

    def get_matrix(self):
        return self._user_defined_matrix

    def adjoint(self, do_queue=False):
        return Unitary(self.matrix.conj().T, qubits=self.qubits, do_queue=do_queue)

    @property
    def eigvals(self):
        return self._eigvals


class IintStateVector(OperatorBase):
    """Initial state preparation (prepared_state.py:29-57): a flat vector of
    2^n amplitudes that replaces |0...0> (pytorch_backend.py:500-510)."""

    _num_params = 0
    _num_qubits = 0

    def __init__(self, matrix, qubits=(), do_queue=True, **kwargs):
        self._user_defined_matrix = np.asarray(matrix)
        super().__init__(qubits=list(qubits), do_queue=do_queue, is_preparation=True, **kwargs)

    def get_matrix(self):
        return self._user_defined_matrix


ops = {"Hadamard", "PauliX", "PauliY", "PauliZ", "I", "S", "T", "SX", "CNOT", "CZ", "CY", "SWAP", "CSWAP",
       "Toffoli", "RX", "RY", "RZ", "Rot", "PhaseShift", "ControlledPhaseShift", "CRX", "CRY", "CRZ", "Unitary"}
obs = {"Hadamard", "PauliX", "PauliY", "PauliZ"}
