"""Benchmark: 20-qubit VQC value+grad circuits/s on one GB300.

Workload (one "step"): a batch of 1024 independent parameter vectors of the
20-qubit ansatz with 10 layers of RX, RY, RZ on every qubit followed by a CNOT
ladder (600 parameters, 790 gates), outputs <Z_i> for every qubit and
<Z_0 Z_1> (21 expectation values), evaluated forward and differentiated with
respect to all 600 parameters (adjoint method), complex64 state.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` is circuits/s with parameters
resident in HBM; ``e2e`` is the same through the public API with the
parameters in pinned host memory and the gradients/outputs copied back every
step.  ``roofline`` is computed from CUDA events around every kernel launch of
the timed region (on the launch stream).  ``--impl reference`` times the
reference algorithm (TeD-Q's per-gate tensordot state-vector loop with torch
autograd, restated in ``oracle/``) on the host CPU cores.
"""

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

# more hardware work queues than the driver's default 8 (before CUDA starts):
# the serving workload's prioritised streams must not share a queue with the
# large circuits' streams
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402
import torch  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "ted-q_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "20q VQC value+grad circuits/s"
UNIT = "circuits/s"

# DRAM bytes per amplitude and pass of the 20-qubit, 10-layer VQC's pass
# kernels, from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum
# of one launch of pass 2 of each sweep at 32 circuits, divided by the
# 32 x 2^20 amplitudes it streams); the bench scales them to its own launches
# for the roofline's "traffic" (the algorithmic figures are 16 and 32).
NCU_DRAM_BYTES_PER_AMP = {"fwd": 14.19, "bwd": 30.17}


def vqc_spec(n, layers, seed=0):
    """Seeded synthetic config-2 circuit (angles drawn uniform[0, 2pi))."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers):
        for q in range(n):
            for name in ("RX", "RY", "RZ"):
                gates.append({"name": name, "qubits": [q], "params": [float(rng.uniform(0, 2 * np.pi))],
                              "trainable": [0]})
        for q in range(n - 1):
            gates.append({"name": "CNOT", "qubits": [q, q + 1], "params": [], "trainable": []})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n)]
    meas.append({"kind": "expval", "list": True,
                 "obs": [{"name": "PauliZ", "qubits": [0]}, {"name": "PauliZ", "qubits": [1]}]})
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


def workload_config(a):
    return {"workload": f"vqc{a.qubits}q_{a.layers}layers_batch{a.batch}",
            "n_qubits": a.qubits, "layers": a.layers, "batch_per_gpu": a.batch,
            "params_per_circuit": 3 * a.qubits * a.layers, "gates": (4 * a.qubits - 1) * a.layers,
            "outputs": f"<Z_i> i<{a.qubits} and <Z_0 Z_1>", "gradient": "adjoint, all parameters",
            "l2": "inputs larger than L2 (state %d MiB per circuit x batch)" % ((8 << a.qubits) >> 20)}


def small8_spec(seed=0):
    """8-qubit hardware-efficient ansatz: 4 layers of RY, RZ on every qubit and
    a CNOT ring i -> i+1 mod 8; <Z_i> on every qubit (64 parameters)."""
    rng = np.random.default_rng(seed)
    n, gates = 8, []
    for _ in range(4):
        for q in range(n):
            for name in ("RY", "RZ"):
                gates.append({"name": name, "qubits": [q], "params": [float(rng.uniform(0, 2 * np.pi))],
                              "trainable": [0]})
        for q in range(n):
            gates.append({"name": "CNOT", "qubits": [q, (q + 1) % n], "params": [], "trainable": []})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(n)]
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


def sv_workload(a):
    """(spec, metric, config, loss) of the state-vector workloads."""
    if a.workload == "small8":
        spec = small8_spec()
        return spec, "8q HEA value+grad circuits/s", {
            "workload": f"hea8q_4layers_ring_batch{a.batch}", "n_qubits": 8, "layers": 4, "batch_per_gpu": a.batch,
            "params_per_circuit": 64, "outputs": "<Z_i> i<8", "gradient": "adjoint, all parameters",
            "l2": "states fit in L2 (2 KiB per circuit); latency-bound"}, "sum"
    if a.workload == "mbl24":
        from tedq_gb300.templates import mbl_spec
        spec = mbl_spec(24, 12, seed=24)
        P = sum(len(g["trainable"]) for g in spec["gates"])
        return spec, "24q MBL 12-layer value+grad circuits/s", {
            "workload": f"mbl24q_12trotter_batch{a.batch}", "n_qubits": 24, "layers": 12, "batch_per_gpu": a.batch,
            "params_per_circuit": P, "gates": len(spec["gates"]), "outputs": "<Z_i> i<24",
            "loss": "sum_i <Z_i>^2", "gradient": "adjoint, all parameters",
            "l2": "inputs larger than L2 (state 128 MiB per circuit x batch)"}, "sumsq"
    return vqc_spec(a.qubits, a.layers), METRIC, workload_config(a), "sum"


# ---------------------------------------------------------------- helpers

def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(rows), "reasons": sorted(reasons)}


def host_info():
    """Host cores and CPU model beside every CPU number."""
    model = platform.processor() or platform.machine()
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return {"threads": torch.get_num_threads(), "cpu_count": os.cpu_count(), "cpu_model": model,
            "torch": torch.__version__}


def dist_setup(backend="nccl"):
    """Replicas: one process per GPU from torchrun's environment; no data-path
    collective (barriers and a max of the timings only)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def replica_seed(base, rank):
    """Each replica draws its own batch (weak scaling)."""
    return base + rank


def aggregate_rate(world, units_per_rank, ms_max):
    """Whole-job throughput: units of all ranks over the slowest rank's time."""
    return world * units_per_rank / (ms_max / 1000.0)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, dev):
    if world == 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU reference

def cpu_reference(spec, n_circuits, seed=1):
    """Reference algorithm on the host: per-gate tensordot loop with torch
    autograd (back_prop), complex64, all host threads.  Returns (circuits/s, secs)."""
    import oracle
    P = sum(len(g["trainable"]) for g in spec["gates"])
    gen = torch.Generator().manual_seed(seed)
    dy = np.ones(len(spec["meas"]))
    t0 = time.perf_counter()
    for _ in range(n_circuits):
        p = torch.rand(P, generator=gen) * 2 * np.pi
        oracle.value_and_grad(spec, p, dy, torch.complex64)
    dt = time.perf_counter() - t0
    return n_circuits / dt, dt


def cpu_sample_size(spec, budget_s):
    rate, dt = cpu_reference(spec, 1)
    return max(1, int(budget_s / max(dt, 1e-3))), rate, dt


def run_reference_arm(a):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    spec = vqc_spec(a.qubits, a.layers)
    threads = torch.get_num_threads()
    k, _, _ = cpu_sample_size(spec, a.cpu_budget / max(1, a.steps))
    k = min(k, 4)
    for _ in range(a.warmup):
        cpu_reference(spec, 1)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        cpu_reference(spec, k)
    dt = time.perf_counter() - t0
    rate = a.steps * k / dt
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * dt / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": workload_config(a),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "host": host_info(),
                             "sample": f"{k} circuit(s) of the workload per step, value+grad by back_prop"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- plain per-circuit GPU path

def plain_gpu_rate(spec, dev, n_circuits=2):
    """The reference's algorithm run per circuit on the GPU with torch ops: one
    tensordot + permute per gate (pytorch_backend.py:358-380), measurements by
    tensordot, gradient by torch autograd.  Returns circuits/s (value+grad)."""
    n = spec["n"]
    gen = torch.Generator().manual_seed(3)
    P = sum(len(g["trainable"]) for g in spec["gates"])

    def one(p):
        k = 0
        state = torch.zeros([2] * n, dtype=torch.complex64, device=dev)
        state.view(-1)[0] = 1
        cnot = torch.tensor([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=torch.complex64,
                            device=dev).reshape(2, 2, 2, 2)
        for g in spec["gates"]:
            q = g["qubits"]
            if g["name"] == "CNOT":
                G = cnot
            else:
                th = p[k:k + 1]
                k += 1
                c, s = torch.cos(th / 2), torch.sin(th / 2)
                z = torch.zeros_like(c)
                if g["name"] == "RX":
                    G = torch.cat([c + 0j, -1j * s, -1j * s, c + 0j]).reshape(2, 2)
                elif g["name"] == "RY":
                    G = torch.cat([c, -s, s, c]).to(torch.complex64).reshape(2, 2)
                else:
                    e = torch.exp(-0.5j * th)
                    G = torch.cat([e, z + 0j, z + 0j, e.conj()]).reshape(2, 2)
            kq = len(q)
            new = torch.tensordot(G, state, (list(range(kq, 2 * kq)), q))
            rest = [x for x in range(n) if x not in q]
            order = list(q) + rest
            state = new.permute([order.index(i) for i in range(n)])
        outs = []
        Z = torch.tensor([[1, 0], [0, -1]], dtype=torch.complex64, device=dev)
        axes = list(range(n))
        for obs in [[o["qubits"][0] for o in m["obs"]] for m in spec["meas"]]:
            ms = state
            for q in obs:
                ms = torch.tensordot(Z, ms, ([1], [q])).permute(list(range(1, q + 1)) + [0] + list(range(q + 1, n)))
            outs.append(torch.tensordot(torch.conj(state), ms, (axes, axes)).real)
        return torch.stack(outs)

    p = (torch.rand(P, generator=gen) * 2 * np.pi).to(dev).requires_grad_(True)
    one(p).sum().backward()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n_circuits):
        p = (torch.rand(P, generator=gen) * 2 * np.pi).to(dev).requires_grad_(True)
        one(p).sum().backward()
    torch.cuda.synchronize()
    return n_circuits / (time.perf_counter() - t0)


# ---------------------------------------------------------------- GPU arm

def run_ours(a):
    world, rank, local = dist_setup()
    dev = torch.device("cuda", torch.cuda.current_device())
    import tedq_gb300 as qai
    from tedq_gb300 import _lib

    spec, metric, config, loss_kind = sv_workload(a)
    t_compile = time.perf_counter()
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", fuse=not a.plain, jit=a.jit,
                                                    tile_qubits=a.tile)
    jit_reason = cc._prog.jit_wait()
    t_compile = time.perf_counter() - t_compile
    info = cc.program_info
    P = cc.num_params
    B = a.batch
    gen = torch.Generator().manual_seed(replica_seed(1000, rank))
    params_host = (torch.rand(a.steps + a.warmup, B, P, generator=gen) * 2 * np.pi)
    params_dev = params_host.to(dev)
    L = _lib.lib()
    h = cc._prog.handle
    stream = torch.cuda.current_stream(dev)

    def loss_of(out):
        return (out * out).sum() if loss_kind == "sumsq" else out.sum()

    def step_dev(i):
        p = params_dev[i].requires_grad_(True)
        out = cc.execute_batch(p)
        loss_of(out).backward()
        return out, p.grad

    for i in range(a.warmup):
        step_dev(i)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    L.tedq_profile_enable(h, 1)
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(a.steps):
        step_dev(a.warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    L.tedq_profile_enable(h, 0)
    prof = _lib.Profile()
    _lib.check(L.tedq_profile_read(h, prof), "tedq_profile_read")
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    value = aggregate_rate(world, B * a.steps, ms)

    # e2e through the public API with host buffers
    ph = params_host.pin_memory()
    for i in range(min(2, a.warmup)):
        p = ph[i].clone().requires_grad_(True)
        out = cc.execute_batch(p)
        loss_of(out).backward()
        out.cpu()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for i in range(a.steps):
        p = ph[a.warmup + i].detach().requires_grad_(True)   # pinned host parameters
        out = cc.execute_batch(p)                             # H2D inside
        loss_of(out).backward()                               # gradients land on the host tensor (D2H)
        res = out.detach().cpu()                              # outputs D2H
        _ = p.grad.numpy()
    f1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms_e2e = max_over_ranks(max(f0.elapsed_time(f1), 1000 * wall), world, dev)
    e2e = world * B * a.steps / (ms_e2e / 1000.0)

    if rank != 0:
        return None

    hbm_peak, peak_kind = read_peaks()
    fam = "bwd" if prof.bwd_ms >= prof.fwd_ms else "fwd"
    launches = getattr(prof, f"{fam}_launches")
    amp_passes = getattr(prof, f"{fam}_amp_passes")
    kms = getattr(prof, f"{fam}_ms")
    bytes_per_amp = 32 if fam == "bwd" else 16
    per_launch_bytes = bytes_per_amp * amp_passes / max(1, launches)
    achieved = per_launch_bytes / (kms / max(1, launches) / 1000.0) / 1e9
    traffic = None
    if a.workload == "vqc" and a.qubits == 20 and a.layers == 10:
        traffic = NCU_DRAM_BYTES_PER_AMP[fam] * amp_passes / max(1, launches)
    gpu_launches = prof.fwd_launches + prof.bwd_launches + prof.meas_launches + prof.lam_launches

    line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64", "data": "synthetic", "config": config,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": B * P * 4,
                    "d2h_bytes_per_step": B * P * 4 + B * info["n_real_outputs"] * 4},
            "gpu_launches": int(gpu_launches),
            "roofline": {"bound": "hbm", "kernel": f"{fam}_pass_kernel", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_kind": peak_kind, "bytes_per_launch": per_launch_bytes,
                         "avg_launch_ms": kms / max(1, launches)},
            "kernels_ms_per_step": {"fwd_pass": prof.fwd_ms / a.steps, "bwd_pass": prof.bwd_ms / a.steps,
                                    "measure": prof.meas_ms / a.steps, "lambda_etc": prof.lam_ms / a.steps},
            "schedule": {k: info[k] for k in ("n_fwd_passes", "n_bwd_passes", "n_fwd_phases", "n_bwd_phases",
                                              "n_fused_gates", "n_elem_gates")},
            "pass_kernels": "generic" if jit_reason else "specialised (NVRTC, sm_103a)",
            "compile_s": round(t_compile, 3),
            "clocks": clk}
    # accuracy of the complex64 results: against this backend's complex128 path
    # on the device (8 circuits of the batch) and, unless --no-cpu, against the
    # complex128 CPU oracle on one circuit (values and gradients)
    try:
        k8 = min(8, B) if a.workload != "mbl24" else min(2, B)
        P8 = params_dev[0][:k8].detach().clone()
        c128 = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", precision="c128", jit=a.jit)
        p32 = P8.clone().requires_grad_(True)
        o32 = cc.execute_batch(p32)
        loss_of(o32).backward()
        p64 = P8.double().requires_grad_(True)
        o64 = c128.execute_batch(p64)
        loss_of(o64).backward()
        acc = {"max_abs_err_vs_c128": float((o32.detach().double() - o64.detach()).abs().max()),
               "max_abs_grad_err_vs_c128": float((p32.grad.double() - p64.grad).abs().max()),
               "circuits": k8}
        if not a.no_cpu and a.workload != "mbl24":
            import oracle
            z = o64.detach()[0].cpu().double()
            dy = (2 * z if loss_kind == "sumsq" else torch.ones_like(z)).numpy()
            v_ref, g_ref = oracle.value_and_grad(spec, P8[0].double().cpu(), dy, torch.complex128)
            acc["max_abs_err_vs_cpu_c128"] = float((o32.detach()[0].cpu().double() - v_ref.reshape(-1)).abs().max())
            acc["max_abs_grad_err_vs_cpu_c128"] = float((p32.grad[0].cpu().double() - g_ref).abs().max())
        line["accuracy"] = acc
    except Exception as e:  # pragma: no cover
        line["accuracy"] = {"error": str(e)[:200]}
    if not a.no_plain and a.workload in ("vqc", "small8"):
        try:
            line["plain_gpu_per_circuit"] = {"value": plain_gpu_rate(spec, dev), "unit": UNIT,
                                             "what": "reference algorithm per circuit with torch ops on the GPU"}
            line["plain_gpu_per_circuit"]["speedup_of_value"] = value / line["plain_gpu_per_circuit"]["value"]
        except Exception as e:  # pragma: no cover
            line["plain_gpu_per_circuit"] = {"error": str(e)[:200]}
    if not a.no_cpu and a.workload == "mbl24":
        # the reference's back_prop keeps every intermediate state (~380 GiB at
        # 24 qubits): time its forward pass, on the first a.mbl_cpu_gates gates
        # (the per-gate tensordot loop costs the same per gate), scaled to all
        import oracle
        ng = len(spec["gates"])
        k = min(ng, a.mbl_cpu_gates) if a.mbl_cpu_gates > 0 else ng
        sub = dict(spec, gates=spec["gates"][:k])
        Pk = sum(len(g["trainable"]) for g in sub["gates"])
        t0 = time.perf_counter()
        oracle.run(sub, torch.rand(Pk, generator=torch.Generator().manual_seed(5)) * 2 * np.pi, torch.complex64)
        dt = (time.perf_counter() - t0) * ng / k
        sample = (f"1 circuit, forward only, {dt:.1f} s" if k == ng else
                  f"forward of the first {k} of {ng} gates of 1 circuit, scaled to all gates: {dt:.1f} s")
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "circuits/s (forward only)",
                                "cores": torch.get_num_threads(), "kind": "port", "host": host_info(),
                                "sample": f"{sample}; back_prop does not fit host memory at 24 qubits"}
    elif not a.no_cpu:
        k, _, _ = cpu_sample_size(spec, a.cpu_budget)
        k = min(k, 8 if a.workload == "vqc" else 256)
        rate, dt = cpu_reference(spec, k)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": torch.get_num_threads(), "kind": "port",
                                "host": host_info(),
                                "sample": f"{k} circuit(s) of the workload, value+grad by back_prop, {dt:.1f} s"}
    return line


# ---------------------------------------------------------------- serving stream

def serving_trace(lam, duration, sizes, depths, rng):
    """Poisson arrivals at ``lam`` req/s for ``duration`` s: (gaps, (n, depth) keys)."""
    n_req = max(20, int(lam * duration))
    gaps = rng.exponential(1.0 / lam, n_req)
    keys = [(sizes[rng.integers(len(sizes))], depths[rng.integers(len(depths))]) for _ in range(n_req)]
    return gaps, keys


def cpu_service_model(sizes, depths, budget_s):
    """Per-request service time of the reference algorithm on the host (the
    oracle's per-gate tensordot loop, value + gradient by back_prop,
    complex64, all host threads) for every (n, depth) of the serving stream.
    n <= 16: measured at the smallest, middle and largest depth, linear in
    depth between; n = 20: measured at the smallest depth and scaled linearly
    in depth (the loop's cost is proportional to the gate count); n = 24:
    the n = 20 time scaled by the state size (16x) and the gate count.
    Returns ({(n, d): seconds}, description)."""
    import oracle
    from tedq_gb300.templates import hea_spec
    gen = torch.Generator().manual_seed(11)

    def one(n, d):
        spec = hea_spec(n, d)
        P = sum(len(g["trainable"]) for g in spec["gates"])
        dy = np.ones(len(spec["meas"]))
        t0 = time.perf_counter()
        oracle.value_and_grad(spec, torch.rand(P, generator=gen) * 2 * np.pi, dy, torch.complex64)
        return time.perf_counter() - t0

    d0, d1, d2 = depths[0], depths[len(depths) // 2], depths[-1]
    model, t_start = {}, time.perf_counter()
    one(4, d0)  # warm-up
    n_gates = lambda n, d: len(hea_spec(n, d)["gates"])  # noqa: E731
    t20 = None
    for n in sizes:
        if n <= 16:
            pts = {d: one(n, d) for d in (d0, d1, d2)}
            for d in depths:
                lo, hi = (d0, d1) if d <= d1 else (d1, d2)
                model[(n, d)] = pts[lo] + (pts[hi] - pts[lo]) * (d - lo) / (hi - lo)
        elif n == 20:
            t20 = one(n, d0)
            for d in depths:
                model[(n, d)] = t20 * d / d0
    for n in sizes:
        if n > 20:
            for d in depths:
                model[(n, d)] = t20 * (2.0 ** (n - 20)) * n_gates(n, d) / n_gates(20, d0)
    desc = (f"reference algorithm per request on the host (oracle port, back_prop, complex64, "
            f"{torch.get_num_threads()} threads): n <= 16 measured at depths {d0}, {d1}, {d2} and interpolated, "
            f"n = 20 measured at depth {d0} and scaled by depth, n = 24 extrapolated from n = 20 by state size and "
            f"gate count; {time.perf_counter() - t_start:.1f} s of measurement; the identical trace replayed "
            f"through a sequential FIFO server with these times")
    return model, desc


def replay_sequential(gaps, keys, service, sizes):
    """One request at a time in arrival order (the reference evaluates one
    circuit per call): throughput and per-bucket latency of the trace."""
    arrive = np.cumsum(gaps)
    free_at = 0.0
    lat = {n: [] for n in sizes}
    for t, k in zip(arrive, keys):
        start = max(t, free_at)
        free_at = start + service[k]
        lat[k[0]].append(1000.0 * (free_at - t))
    per = {str(n): {"count": len(v), "p50_ms": float(np.percentile(v, 50)) if v else None,
                    "p99_ms": float(np.percentile(v, 99)) if v else None} for n, v in lat.items()}
    return {"throughput_req_s": len(keys) / (free_at - arrive[0] + 1e-12), "per_qubits": per}


def run_serving(a):
    """Serving stream: Poisson arrivals of value+grad evaluations of the
    hardware-efficient ansatz, n uniform over {4,8,12,16,20,24}, depth uniform
    in [2, 12], swept over arrival rates; throughput and p50/p99 latency per
    qubit bucket.  Specialised kernels compile in the background while the
    generic kernels serve.  Size-class lanes: n <= 16 on high-priority streams
    with reserved memory.  The CPU baseline replays the identical trace through
    the reference algorithm one request at a time."""
    import threading
    import tedq_gb300 as qai
    from tedq_gb300.serving import Server
    from tedq_gb300.templates import hea_spec
    torch.cuda.set_device(0)
    sizes, depths = [4, 8, 12, 16, 20, 24], list(range(2, 13))
    progs = {(n, d): qai.Circuit.from_spec(hea_spec(n, d)).compilecircuit(backend="gb300", jit=2)
             for n in sizes for d in depths}
    rates = [float(r) for r in a.rates.split(",")]
    traces = {lam: serving_trace(lam, a.duration, sizes, depths, np.random.default_rng(2024 + int(lam)))
              for lam in rates}
    results = []
    t_gpu = time.perf_counter()
    # a server takes traffic with its programs compiled: wait for the
    # specialised kernels of every program (compiled in the background on
    # host threads), so that none is loaded in the middle of the sweep
    t_jit = time.perf_counter()
    for cc in progs.values():
        cc._prog.jit_wait()
    t_jit = time.perf_counter() - t_jit
    with Server(max_batch=64, max_wait_us=300, memory_budget_bytes=int(a.budget_gb * (1 << 30)),
                n_streams=8, lane_qubits=a.lane_qubits) as srv:
        # warm-up: every program twice (loads its modules, touches the arena)
        for _ in range(2):
            for cc in progs.values():
                srv.wait(srv.submit(cc, np.zeros(cc.num_params, np.float32)), timeout_s=600)
        rng = np.random.default_rng(7)
        for lam in rates:
            gaps, keys = traces[lam]
            n_req = len(keys)
            params = [rng.uniform(0, 2 * np.pi, progs[k].num_params).astype(np.float32) for k in keys]
            tickets = [None] * n_req
            t0 = time.perf_counter()

            def producer():
                t = t0
                for i in range(n_req):
                    t += gaps[i]
                    d = t - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    tickets[i] = srv.submit(progs[keys[i]], params[i])
            th = threading.Thread(target=producer)
            th.start()
            lat = {n: [] for n in sizes}
            done_at = t0
            for i in range(n_req):
                while tickets[i] is None:
                    time.sleep(0.0002)
                _, _, info = srv.wait(tickets[i], timeout_s=600)
                lat[keys[i][0]].append(info["total_us"] / 1000.0)
                done_at = max(done_at, time.perf_counter())
            th.join()
            wall = done_at - t0
            per = {str(n): {"count": len(v), "p50_ms": float(np.percentile(v, 50)) if v else None,
                            "p99_ms": float(np.percentile(v, 99)) if v else None} for n, v in lat.items()}
            results.append({"offered_req_s": lam, "requests": n_req, "throughput_req_s": n_req / wall,
                            "per_qubits": per})
        stats = srv.stats()
    t_gpu = time.perf_counter() - t_gpu
    top = max(r["throughput_req_s"] for r in results)
    line = {"metric": "serving value+grad requests/s (mixed n 4-24, HEA depth 2-12); p50/p99 ms per qubit bucket",
            "value": top, "unit": "requests/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": "serving_stream_poisson", "rates_req_s": rates, "duration_s": a.duration,
                       "qubits": sizes, "depth": [2, 12], "memory_budget_gb": a.budget_gb, "max_batch": 64,
                       "n_streams": 8, "lane_qubits": a.lane_qubits if a.lane_qubits else 16},
            "e2e": {"value": top, "unit": "requests/s",
                    "what": "requests submitted from host memory, results and gradients returned to host memory"},
            "sweep": results, "server": stats, "gpu_wall_s": round(t_gpu, 1), "compile_wait_s": round(t_jit, 1)}
    if not a.no_cpu:
        model, desc = cpu_service_model(sizes, depths, a.cpu_budget)
        replays = [dict(offered_req_s=lam, **replay_sequential(*traces[lam], model, sizes)) for lam in rates]
        line["cpu_baseline"] = {"value": replays[-1]["throughput_req_s"], "unit": "requests/s",
                                "cores": torch.get_num_threads(), "kind": "port", "host": host_info(),
                                "sample": desc, "sweep": replays}
    return line


# ---------------------------------------------------------------- tensor-network workload

TN_METRIC = "6x6 lattice 8-layer centre <Z> tensor-network contractions/s"


def tn_params(rows, cols, layers, count, seed):
    """Haar-random Rot angles, [count, layers * rows * cols * 3]."""
    from tedq_gb300.templates import lattice_params
    return np.stack([lattice_params(rows, cols, layers, seed * 100003 + i) for i in range(count)])


def tn_cpu_rate(spec, prm_rows, dtype):
    """Reference TN algorithm on the host (sandwich network, greedy pairwise
    order, tensordot contractions; oracle/tn_oracle.py).  The order is computed
    once outside the timed loop, as the reference's contract_expression does."""
    from oracle import tn_oracle
    arrays, idx = tn_oracle.network(spec, list(prm_rows[0]))
    order = tn_oracle.greedy_order(idx)
    t0 = time.perf_counter()
    vals = []
    for row in prm_rows:
        arrays, idx = tn_oracle.network(spec, list(row))
        vals.append(tn_oracle.contract(arrays, idx, order, dtype).real)
    dt = time.perf_counter() - t0
    return len(prm_rows) / dt, dt, np.array(vals)


def run_tn(a):
    world, rank, local = dist_setup()
    dev = torch.device("cuda", torch.cuda.current_device())
    import tedq_gb300 as qai
    from tedq_gb300 import _lib
    from tedq_gb300.templates import lattice_spec

    R, C, Lr = 6, 6, 8
    spec = lattice_spec(R, C, Lr, seed=0)
    B = a.batch
    t_plan = time.perf_counter()
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", tn_mode=True, tn_gemm=a.tn_gemm,
                                                    tn_graphs=bool(a.tn_graphs), requires_grad=False)
    t_plan = time.perf_counter() - t_plan
    info = cc.program_info
    P = info["n_params"]
    params_host = torch.tensor(tn_params(R, C, Lr, (a.steps + a.warmup) * B, 1000 + rank),
                               dtype=torch.float32).reshape(a.steps + a.warmup, B, P)
    params_dev = params_host.to(dev)
    outs = [torch.empty((B, 1), dtype=torch.float32, device=dev) for _ in range(a.steps + a.warmup)]
    L = _lib.lib()
    prog = cc._prog
    stream = torch.cuda.current_stream(dev)
    ws, wsb = cc._ws.get(prog.workspace_bytes(B), dev)

    def step(i):  # the public C entry point on device-resident buffers (graph replay after the 2nd call)
        _lib.check(L.tedq_tn_contract(prog.handle, ctypes.c_void_p(params_dev[i].data_ptr()), B,
                                      ctypes.c_void_p(outs[i].data_ptr()), ctypes.c_void_p(ws), wsb,
                                      ctypes.c_void_p(stream.cuda_stream)), "tedq_tn_contract")

    # every timed step uses its own parameter and output buffers; with graphs,
    # capture each one during warm-up (two calls per buffer set: eager, captured)
    for i in range(a.warmup + a.steps):
        step(i)
        if a.tn_graphs:
            step(i)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(a.steps):
        step(a.warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    value = world * B * a.steps / (ms / 1000.0)

    # kernel timing: events around every launch (eager, same workload)
    L.tedq_tn_profile_enable(prog.handle, 1)
    for i in range(a.steps):
        step(a.warmup + i)
    torch.cuda.synchronize()
    L.tedq_tn_profile_enable(prog.handle, 0)
    prof = _lib.TnProfile()
    _lib.check(L.tedq_tn_profile_read(prog.handle, ctypes.byref(prof)), "tedq_tn_profile_read")

    # e2e through the public API: pinned host parameters in, host results out
    ph = params_host.pin_memory()
    for i in range(min(2, a.warmup)):
        cc.execute_batch(ph[i]).cpu()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for i in range(a.steps):
        res = cc.execute_batch(ph[a.warmup + i]).cpu()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms_e2e = max_over_ranks(1000 * wall, world, dev)
    e2e = world * B * a.steps / (ms_e2e / 1000.0)

    if rank != 0:
        return None
    # accuracy: complex64 (this GEMM mode) against complex128 on the device and the CPU oracle
    ref = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", tn_mode=True, precision="c128",
                                                      requires_grad=False)
    v128 = ref.execute_batch(params_dev[0].double()).cpu().numpy()[:, 0]
    v64 = outs[0].cpu().numpy()[:, 0]
    peak_kind = "measured"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
    except Exception:
        bf16, peak_kind = 1900.0, "fallback"
    if a.tn_gemm in ("tc32", "auto"):
        peak = bf16 / 2.0 / 3.0
        peak_kind += (" bf16 dense / 2 (TF32 rate) / 3 (each FP32-accurate product is three TF32 "
                      "tensor-core products)")
    elif a.tn_gemm == "tf32":
        peak = bf16 / 2.0
        peak_kind += " bf16 dense / 2 (TF32 rate)"
    else:
        peak = None
        peak_kind = "FP32 SIMT (no tensor-core peak)"
    # the dominant kernel: the tensor-core GEMMs when they run, else every
    # contraction launch
    tc = prof.tc_ms > 0
    achieved = (prof.tc_flops / (prof.tc_ms / 1000.0) / 1e12 if tc else
                prof.gemm_flops / (prof.gemm_ms / 1000.0) / 1e12 if prof.gemm_ms else 0.0)
    per_call = prof.leaf_launches + prof.gather_launches + prof.gemm_launches + prof.root_launches
    line = {"metric": TN_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": f"c64 ({a.tn_gemm} GEMM, FP32 accumulate)", "data": "synthetic",
            "config": {"workload": f"tn_lattice{R}x{C}_{Lr}layers_centreZ_batch{B}", "sites": R * C, "layers": Lr,
                       "gates": len(spec["gates"]), "gates_in_light_cone": info["gates_kept"],
                       "params_per_circuit": P, "contractions_per_circuit": info["n_steps"],
                       "largest_intermediate_log2": info["max_rank"], "sliced": info["n_sliced"],
                       "flops_per_circuit": 2.0 ** info["log2_flops"], "batch_per_gpu": B,
                       "plan_s": round(t_plan, 3), "graphs": bool(a.tn_graphs),
                       "l2": "inputs larger than L2 (intermediates %.1f GB per step)" %
                             (prog.workspace_bytes(B) / 1e9)},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": B * P * 4, "d2h_bytes_per_step": B * 4},
            "gpu_launches": int(per_call),
            "roofline": {"bound": "tensor",
                         "kernel": ("tn_gemm_tc_kernel (tcgen05 kind::tf32, 3xTF32 split; 4M real embedding)" if tc
                                    else "contractions: level launches + FMA GEMMs"),
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if peak else None, "traffic": None, "peak_kind": peak_kind,
                         "tc_gemm_launches_per_step": prof.tc_launches / a.steps,
                         "tc_gemm_ms_per_step": prof.tc_ms / a.steps,
                         "contractions_tflops": (prof.gemm_flops / (prof.gemm_ms / 1000.0) / 1e12
                                                 if prof.gemm_ms else 0.0),
                         "gemm_ms_per_step": prof.gemm_ms / a.steps, "gather_ms_per_step": prof.gather_ms / a.steps,
                         "gather_gbs": prof.gather_bytes / (prof.gather_ms / 1000.0) / 1e9 if prof.gather_ms else 0,
                         "leaf_ms_per_step": prof.leaf_ms / a.steps, "root_ms_per_step": prof.root_ms / a.steps,
                         "launches_per_step": per_call / a.steps},
            "accuracy": {"max_abs_err_vs_c128": float(np.abs(v64 - v128).max())},
            "clocks": clk}
    if not a.no_cpu:
        rows = params_host[0, : max(1, a.tn_cpu_circuits)].double().numpy()
        rate, dt, vcpu = tn_cpu_rate(spec, rows, np.complex64)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": torch.get_num_threads(), "kind": "port",
                                "host": host_info(),
                                "sample": f"{len(rows)} circuit(s), complex64 tensordot contractions, {dt:.1f} s"}
        _, _, v128cpu = tn_cpu_rate(spec, rows[:2], np.complex128)
        line["accuracy"]["max_abs_err_vs_cpu_c128"] = float(np.abs(v64[:2] - v128cpu).max())
    return line


WORKLOAD_SETTINGS = {
    # per-workload settings of the default run's "workloads" entries (each a
    # compact line of its own: value, e2e, roofline, cpu_baseline)
    # specialised kernels for the 8-qubit circuit too (the automatic mode
    # compiles them from 14 qubits on; jit=1 asks for them, as a training
    # loop over a small circuit would): 5.3 M against 4.3 M circuits/s
    "small8": {"batch": 4096, "steps": 20, "warmup": 3, "cpu_budget": 5.0, "jit": 1},
    "mbl24": {"batch": 256, "steps": 2, "warmup": 3, "mbl_cpu_gates": 150},
    "tn": {"batch": 1024, "steps": 10, "warmup": 3, "tn_cpu_circuits": 32},
    "serving": {"rates": "100,500,1000", "duration": 2.0},
}
ENTRY_KEYS = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "dtype", "config", "e2e",
              "gpu_launches", "roofline", "cpu_baseline", "accuracy", "plain_gpu_per_circuit", "sweep", "clocks",
              "kernels_ms_per_step", "pass_kernels")


def run_workloads(a):
    """The other benchmark configurations, each with its own settings, for the
    default (N=1) run: 8-qubit HEA, 24-qubit MBL, the tensor-network lattice
    and the serving stream."""
    out = {}
    for name in [w for w in a.workloads.split(",") if w]:
        b = argparse.Namespace(**vars(a))
        b.workload = name
        b.no_plain = name != "small8"
        for k, v in WORKLOAD_SETTINGS.get(name, {}).items():
            setattr(b, k, v)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        t0 = time.perf_counter()
        try:
            line = run_serving(b) if name == "serving" else run_tn(b) if name == "tn" else run_ours(b)
            entry = {k: line[k] for k in ENTRY_KEYS if k in line}
        except Exception as e:  # pragma: no cover - reported, not fatal for the headline
            entry = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
        entry["wall_s"] = round(time.perf_counter() - t0, 1)
        out[name] = entry
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=20)
    ap.add_argument("--layers", type=int, default=10)
    ap.add_argument("--batch", type=int, default=None, help="circuits per step (default 4096 for small8, else 1024)")
    ap.add_argument("--plain", action="store_true", help="unfused per-gate passes")
    ap.add_argument("--jit", type=int, default=0, help="specialised kernels: 0 auto, 1 on, -1 off")
    ap.add_argument("--tile", type=int, default=0, help="forward tile qubits (0 = default)")
    ap.add_argument("--workload", default="vqc", choices=["vqc", "small8", "mbl24", "serving", "tn"])
    ap.add_argument("--workloads", default="small8,mbl24,tn,serving",
                    help="with the default vqc workload at N=1: the other configurations to run after it "
                         "(each reported under 'workloads'); empty = none")
    ap.add_argument("--tn-gemm", default="auto", choices=["tc32", "tf32", "fp32", "auto"])
    ap.add_argument("--tn-cpu-circuits", type=int, default=64)
    ap.add_argument("--tn-graphs", type=int, default=0, help="replay each call as a CUDA graph")
    ap.add_argument("--rates", default="100,500,2000,5000")
    ap.add_argument("--duration", type=float, default=2.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--lane-qubits", type=int, default=0, help="serving lanes: 0 = 16, < 0 = one lane")
    ap.add_argument("--mbl-cpu-gates", type=int, default=0,
                    help="mbl24 CPU baseline: time the forward of this many gates and scale (0 = all)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    a = ap.parse_args()
    if a.batch is None:
        a.batch = 4096 if a.workload == "small8" else 1024
    if a.impl == "reference":
        return run_reference_arm(a)
    if a.workload == "serving":
        line = run_serving(a)
    elif a.workload == "tn":
        line = run_tn(a)
    else:
        line = run_ours(a)
    if line is None:  # ranks other than 0
        return 0
    if a.workload == "vqc" and line.get("n_gpus", 1) == 1 and a.workloads:
        line["workloads"] = run_workloads(a)
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
