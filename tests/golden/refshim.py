"""Import the unmodified reference TeD-Q in a container that has its checkout.

Test infrastructure: ``import_reference(path)`` puts stub modules for the
reference's optional dependencies that are not installed here (jax, qiskit,
quafu, matplotlib, panel, IPython, toolz, ray, cotengra) into the import
system, adds the checkout to ``sys.path`` and returns the ``tedq`` package.
Nothing of the reference is copied; the stubs only satisfy its unconditional
imports (tedq/backends/__init__.py:7-10, tedq/__init__.py:5-8,
tensor_network.py:27).  Used by the fixture generator, the port calibration
and the CPU tests that exercise the reference's own objects.
"""

import importlib.abc
import importlib.machinery
import os
import sys
import types
import warnings

import numpy as np

DEFAULT_PATH = "/root/reference"

_STUB_ROOTS = {"jax", "jaxlib", "qiskit", "quafu", "matplotlib", "panel", "IPython",
               "toolz", "ray", "cotengra", "qiskit_ibm_provider"}


class _Stub(types.ModuleType):
    __path__ = []

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        full = self.__name__ + "." + name
        if full not in sys.modules:
            sys.modules[full] = _Stub(full)
        return sys.modules[full]

    def __call__(self, *a, **k):
        return _Stub("call")

    def __mro_entries__(self, bases):
        return (object,)


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in _STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        if spec.name == "jax.numpy":
            return np
        return _Stub(spec.name)

    def exec_module(self, module):
        pass


def available(path=DEFAULT_PATH):
    return os.path.isdir(os.path.join(path, "tedq"))


def import_reference(path=DEFAULT_PATH):
    """The reference's ``tedq`` package (imported once per process)."""
    if "tedq" in sys.modules and getattr(sys.modules["tedq"], "__file__", "").startswith(path):
        return sys.modules["tedq"]
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _StubFinder())
    if path not in sys.path:
        sys.path.insert(0, path)
    warnings.filterwarnings("ignore")
    import tedq  # noqa: F401
    import tedq.backends.pytorch_backend  # noqa: F401
    return sys.modules["tedq"]


def record_circuit(tq, case, rdtype, param_shape=()):
    """Record a fixture case (the dict format of tests/golden: ``n``,
    ``gates``, ``meas``, ``init_state``) with the reference's own circuit API
    (``tq`` = the reference's ``tedq``); gate parameters become tensors of
    ``param_shape`` (0-d by default) and ``rdtype``."""
    import torch

    def circuit_def(*_):
        if case.get("init_state") is not None:
            a = np.asarray(case["init_state"])
            tq.IintStateVector(a[:, 0] + 1j * a[:, 1], qubits=[])
        for gg in case["gates"]:
            cls = getattr(tq, gg["name"])
            pars = [torch.full(param_shape, p, dtype=rdtype) for p in gg["params"]]
            op = cls(*pars, qubits=gg["qubits"], trainable_params=gg["trainable"])
            if gg.get("inv"):
                op.inverse()
        out = []
        for m in case["meas"]:
            if m["kind"] == "expval":
                obs = [getattr(tq, o["name"])(qubits=o["qubits"]) for o in m["obs"]]
                out.append(tq.expval(obs if m["list"] else obs[0]))
            elif m["kind"] == "probs":
                pm = tq.probs(qubits=m["qubits"])
                # the reference's probs() accepts after_state but does not pass
                # it on (measurement.py:174-207); the measurement object carries
                # the flag that execute reads (pytorch_backend.py:474)
                pm.after_state = bool(m.get("after_state", False))
                out.append(pm)
            else:
                out.append(tq.state())
        return out
    return tq.Circuit(circuit_def, case["n"])
