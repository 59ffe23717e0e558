"""Continuous-batching evaluation server (wraps ``tedq_server_*``).

The reference evaluates one circuit per call (``PyTorchBackend.__call__``,
tedq/backends/pytorch_backend.py:124-165) and spreads a dataset over devices
with ``torch.nn.DataParallel`` in its QUDIO backend
(tedq/backends/qudio_backend.py:45-124).  ``Server`` instead keeps compiled
programs and device memory resident and lets requests for any compiled
circuit arrive at any time: a native worker thread batches queued requests of
the same circuit, runs forward and adjoint on its own streams while other
batches are in flight, and admits new batches as the memory budget frees up.
"""

import ctypes

import numpy as np

from . import _lib


class RequestError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


class Server:
    def __init__(self, device=0, n_streams=4, max_batch=256, max_wait_us=200, memory_budget_bytes=1 << 30,
                 paused=False, lane_qubits=0):
        """``lane_qubits``: states of at most this many qubits are served in
        the small lane (own high-priority streams and a reserved part of the
        budget); 0 = 16, a negative value = one lane for every request."""
        L = _lib.lib()
        o = _lib.ServerOptions()
        o.device, o.n_streams, o.max_batch, o.max_wait_us = device, n_streams, max_batch, max_wait_us
        o.memory_budget_bytes = int(memory_budget_bytes)
        o.paused = 1 if paused else 0
        o.lane_qubits = int(lane_qubits)
        h = ctypes.c_void_p()
        _lib.check(L.tedq_server_create(ctypes.byref(o), ctypes.byref(h)), "tedq_server_create")
        self._h = h
        self._meta = {}

    def submit(self, compiled, params, dy=None, with_grad=True):
        """Queue one evaluation of ``compiled`` (a GB300Backend) at ``params``;
        returns a ticket."""
        prog = compiled._prog
        dt = np.float64 if prog.precision == "c128" else np.float32
        p = np.ascontiguousarray(np.asarray(params, dtype=dt).reshape(-1))
        if p.size != prog.n_params:
            raise ValueError(f"expected {prog.n_params} parameters, got {p.size}")
        d = None if dy is None else np.ascontiguousarray(np.asarray(dy, dtype=dt).reshape(-1))
        t = ctypes.c_int64()
        _lib.check(_lib.lib().tedq_server_submit(self._h, prog.handle, p.ctypes.data_as(ctypes.c_void_p),
                                                 None if d is None else d.ctypes.data_as(ctypes.c_void_p),
                                                 1 if with_grad else 0, ctypes.byref(t)), "tedq_server_submit")
        self._meta[t.value] = (prog.n_real, prog.n_params, dt, with_grad)
        return t.value

    def wait(self, ticket, timeout_s=None):
        """(outputs, gradient or None, info) of a finished request; raises
        TimeoutError when ``timeout_s`` expires, RequestError when it failed."""
        n_real, n_params, dt, with_grad = self._meta[ticket]
        out = np.empty(n_real, dtype=dt)
        grad = np.empty(n_params, dtype=dt) if with_grad else None
        res = _lib.RequestResult()
        st = _lib.lib().tedq_server_wait(self._h, ticket, -1 if timeout_s is None else int(timeout_s * 1e6),
                                         out.ctypes.data_as(ctypes.c_void_p),
                                         None if grad is None else grad.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.byref(res))
        if st == _lib.ERR_TIMEOUT:
            raise TimeoutError(_lib.last_error())
        self._meta.pop(ticket, None)
        if st != _lib.OK:
            raise RequestError(st, _lib.last_error())
        return out, grad, {"batch_size": res.batch_size, "queue_us": res.queue_us, "total_us": res.total_us}

    def cancel(self, ticket):
        _lib.check(_lib.lib().tedq_server_cancel(self._h, ticket), "tedq_server_cancel")

    def resume(self):
        _lib.check(_lib.lib().tedq_server_resume(self._h), "tedq_server_resume")

    def stats(self):
        s = _lib.ServerStats()
        _lib.check(_lib.lib().tedq_server_stats(self._h, ctypes.byref(s)), "tedq_server_stats")
        return {f: getattr(s, f) for f, _ in s._fields_ if f != "reserved"}

    def close(self):
        if self._h is not None and self._h.value:
            _lib.lib().tedq_server_destroy(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
