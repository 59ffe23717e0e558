"""NumPy executor of an exported tensor-network plan (``tedq_tn_plan_describe``).

Runs exactly what the device runs -- per step the two bit-permutation gathers
into planar real operands (with the complex combination of a producer's real
product), one real GEMM [Re A; Im A] (2M x K) x [Re B, Im B]^T (K x 2N), and the
root value P(0,0) - P(1,1) summed over slices -- in float64, so the plan's
index maps, slicing offsets and 4M block layout are checked on the CPU.
Parameter-dependent gate tensors come from the oracle's gate definitions.
"""

import numpy as np
import torch

import oracle.sv_oracle as so

_OP_NAMES = {14: "RX", 15: "RY", 16: "RZ", 17: "Rot", 18: "PhaseShift", 19: "ControlledPhaseShift",
             20: "CRX", 21: "CRY", 22: "CRZ"}


def _param_matrix(g, prm):
    pars = []
    for j in range(3 if g["op"] == 17 else 1):
        v = prm[g["slot"][j]] if g["slot"][j] >= 0 else g["val"][j]
        pars.append(torch.tensor([float(v)], dtype=torch.float64))
    t = so._gate_tensor_trainable(_OP_NAMES[g["op"]], pars, torch.complex128)
    return t.reshape(-1).numpy()


def _leaf(net, t, prm):
    T = net["tensors"][t]
    size = 1 << len(T["full_idx"])
    if T["batched"]:
        m = _param_matrix(net["gates"][T["gate"]], prm)
        return np.conj(m) if T["leaf"] == 3 else m
    c = np.asarray(net["constants"][2 * T["off"]: 2 * (T["off"] + size)], dtype=np.float64)
    return c[0::2] + 1j * c[1::2]


def _gather(net, op, store, sl):
    T = net["tensors"][op["tensor"]]
    nbits = op["nf"] + op["nc"]
    e = np.arange(1 << nbits, dtype=np.int64)
    flat = np.zeros_like(e)
    for q, bit in op["slice_bit"]:
        flat += ((sl >> q) & 1) << bit
    for j, bit in enumerate(op["src_bit"]):
        flat += ((e >> j) & 1) << bit
    src = store[op["tensor"]]
    if T["leaf"] >= 0:
        vals = src[flat]
    else:
        M, N = 1 << T["lm"], 1 << T["ln"]
        i, j = flat >> T["ln"], flat & (N - 1)
        vals = (src[i, j] - src[M + i, N + j]) + 1j * (src[i, N + j] + src[M + i, j])
    F, K = 1 << op["nf"], 1 << op["nc"]
    v = vals.reshape(F, K)
    return np.concatenate([v.real, v.imag], axis=0)  # [2F, K]


def run_net(net, prm):
    """Expectation value of one network for one parameter vector."""
    leaves = {t: _leaf(net, t, prm) for t in range(net["n_leaves"])}
    total = 0.0
    for sl in range(1 << len(net["sliced"])):
        store = dict(leaves)
        for st in net["steps"]:
            A = _gather(net, st["opa"], store, sl)
            B = _gather(net, st["opb"], store, sl)
            store[st["out"]] = A @ B.T  # P: [2M, 2N]
        P = store[net["root"]]
        total += P[0, 0] - P[1, 1]
    return total


def run(desc, prm):
    return np.array([run_net(net, np.asarray(prm, dtype=np.float64)) for net in desc["nets"]])


def check_arenas(net):
    """Live intermediates never overlap in their arena (batched and unbatched
    separately); the output of a step may reuse the space of its inputs."""
    T = net["tensors"]
    L = net["n_leaves"]
    live = {}
    for st in net["steps"]:
        for t in (st["a"], st["b"]):
            if t >= L:
                live.pop(t)
        o = st["out"]
        size = 4 << (T[o]["lm"] + T[o]["ln"])
        lo, hi = T[o]["arena"], T[o]["arena"] + size
        arena_max = net["batched_arena"] if T[o]["batched"] else net["unbatched_arena"]
        assert 0 <= lo and hi <= arena_max
        for t, (b, l2, h2) in live.items():
            if b == T[o]["batched"]:
                assert hi <= l2 or h2 <= lo, f"tensor {o} overlaps live tensor {t}"
        live[o] = (T[o]["batched"], lo, hi)
    assert list(live) == [net["root"]]
