"""Serving loop (continuous batching): each result equals the same circuit
evaluated alone, with requests of several circuits in the mix; bounded waits,
cancellation, shutdown and budget rejection fail on the host with status codes."""

import threading
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402
from tedq_gb300.serving import RequestError, Server  # noqa: E402
from tedq_gb300.templates import hea_spec  # noqa: E402

DEV = "cuda:0"


def _compile(n, depth):
    return qai.Circuit.from_spec(hea_spec(n, depth)).compilecircuit(backend="gb300")


def _alone(cc, params):
    p = torch.tensor(params, dtype=torch.float32, device=DEV).reshape(1, -1).requires_grad_(True)
    out = cc.execute_batch(p)
    out.sum().backward()
    return out[0].detach().cpu().numpy(), p.grad[0].cpu().numpy()


def test_mixed_requests_equal_alone_and_batch():
    progs = {k: _compile(*k) for k in [(4, 2), (8, 3), (12, 2)]}
    rng = np.random.default_rng(0)
    jobs = []
    with Server(max_batch=64, memory_budget_bytes=256 << 20, paused=True) as srv:
        for i in range(5):
            for k, cc in progs.items():
                p = rng.uniform(0, 2 * np.pi, cc.num_params).astype(np.float32)
                jobs.append((k, p, srv.submit(cc, p)))
        srv.resume()
        for k, p, t in jobs:
            out, grad, info = srv.wait(t, timeout_s=60)
            assert info["batch_size"] == 5
            want_out, want_grad = _alone(progs[k], p)
            np.testing.assert_allclose(out, want_out, atol=1e-5, rtol=1e-5)
            np.testing.assert_allclose(grad, want_grad, atol=1e-5, rtol=1e-5)
        st = srv.stats()
        assert st["completed"] == 15 and st["batches"] == 3 and st["in_flight_bytes"] == 0


def test_continuous_arrivals():
    progs = [_compile(6, 2), _compile(10, 3), _compile(14, 2)]
    rng = np.random.default_rng(1)
    submitted = []
    with Server(max_batch=16, max_wait_us=100, memory_budget_bytes=256 << 20) as srv:
        def producer():
            for i in range(40):
                cc = progs[i % 3]
                p = rng.uniform(0, 2 * np.pi, cc.num_params).astype(np.float32)
                submitted.append((cc, p, srv.submit(cc, p)))
                time.sleep(0.0005 * (i % 4))
        th = threading.Thread(target=producer)
        th.start()
        th.join()
        for cc, p, t in submitted:
            out, grad, info = srv.wait(t, timeout_s=60)
            want_out, want_grad = _alone(cc, p)
            np.testing.assert_allclose(out, want_out, atol=1e-5, rtol=1e-5)
            np.testing.assert_allclose(grad, want_grad, atol=1e-5, rtol=1e-5)
            assert info["total_us"] >= info["queue_us"] >= 0
        assert srv.stats()["completed"] == 40


def test_timeout_cancel_and_shutdown():
    cc = _compile(6, 2)
    p = np.zeros(cc.num_params, dtype=np.float32)
    srv = Server(paused=True, memory_budget_bytes=64 << 20)
    t1 = srv.submit(cc, p)
    with pytest.raises(TimeoutError):
        srv.wait(t1, timeout_s=0.02)
    srv.cancel(t1)
    with pytest.raises(RequestError) as e:
        srv.wait(t1, timeout_s=1)
    assert e.value.status == _lib.ERR_STATE
    srv.submit(cc, p)
    srv.close()  # queued request fails with TEDQ_ERR_STATE; no hang


def test_request_beyond_budget_is_rejected():
    cc = _compile(16, 1)  # psi + lambda = 1 MiB per circuit
    with Server(memory_budget_bytes=1 << 20) as srv:
        t = srv.submit(cc, np.zeros(cc.num_params, dtype=np.float32))
        with pytest.raises(RequestError) as e:
            srv.wait(t, timeout_s=30)
        assert e.value.status == _lib.ERR_OOM


def test_submit_wrong_parameter_count():
    cc = _compile(4, 1)
    with Server(memory_budget_bytes=16 << 20) as srv:
        with pytest.raises(ValueError):
            srv.submit(cc, np.zeros(cc.num_params + 1, dtype=np.float32))


def test_kernel_limits_shared_across_threads():
    """A small circuit run on another host thread must not lower the shared-
    memory limit a larger circuit needs on this thread."""
    big = _compile(13, 1)
    small = _compile(4, 1)
    big.execute_batch(torch.zeros(1, big.num_params, device=DEV))
    th = threading.Thread(target=lambda: small.execute_batch(torch.zeros(1, small.num_params, device=DEV)))
    th.start()
    th.join()
    out = big.execute_batch(torch.zeros(2, big.num_params, device=DEV))
    torch.cuda.synchronize()
    assert torch.allclose(out, torch.ones_like(out))


def test_small_request_not_blocked_by_large_batches():
    """Size-class lanes: a 4-qubit request submitted while 24-qubit batches
    hold the large lane's streams and memory completes before those batches
    do (its own high-priority stream and reserved memory), with the result it
    has alone."""
    big, small = _compile(24, 8), _compile(4, 2)
    rng = np.random.default_rng(3)
    with Server(n_streams=4, max_batch=32, max_wait_us=100, memory_budget_bytes=16 << 30) as srv:
        for cc in (big, small):  # warm-up: compile and load the kernels
            srv.wait(srv.submit(cc, np.zeros(cc.num_params, dtype=np.float32)), timeout_s=300)
        bigs = [srv.submit(big, rng.uniform(0, 2 * np.pi, big.num_params).astype(np.float32)) for _ in range(64)]
        time.sleep(0.02)
        p = rng.uniform(0, 2 * np.pi, small.num_params).astype(np.float32)
        out, grad, info = srv.wait(srv.submit(small, p), timeout_s=60)
        with pytest.raises(TimeoutError):  # the large batches are still running
            srv.wait(bigs[-1], timeout_s=0)
        want_out, want_grad = _alone(small, p)
        np.testing.assert_allclose(out, want_out, atol=1e-5, rtol=1e-5)
        np.testing.assert_allclose(grad, want_grad, atol=1e-5, rtol=1e-5)
        for t in bigs:
            srv.wait(t, timeout_s=300)
        assert srv.stats()["completed"] == 64 + 3
