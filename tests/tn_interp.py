"""NumPy executor of an exported tensor-network plan (``tedq_tn_plan_describe``).

Runs exactly what the device runs -- per step the two bit-permutation gathers
into rows of real GEMM operands (the operand with the smaller free dimension
in the doubled [[Re, -Im], [Im, Re]] form of the real embedding), one real GEMM
whose column-major result holds Re C and Im C ("planar" or "split" layout), and
the root's real part summed over slices -- in float64, so the plan's index
maps, slicing offsets and GEMM layouts are checked on the CPU.
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


def _complex(net, op, store, sl):
    """Operand values as a complex [F, K] array (rows: free index, columns:
    contracted index), read through the step's bit map."""
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
        i, j = flat & (M - 1), flat >> T["lm"]
        sj, sp = (2 * M, M) if T["split"] else (M, M * N)
        vals = src[j * sj + i] + 1j * src[j * sj + i + sp]
    return vals.reshape(1 << op["nf"], 1 << op["nc"])


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
        i, j = flat & (M - 1), flat >> T["lm"]
        sj, sp = (2 * M, M) if T["split"] else (M, M * N)
        vals = src[j * sj + i] + 1j * src[j * sj + i + sp]
    F, K = 1 << op["nf"], 1 << op["nc"]
    v = vals.reshape(F, K)
    rows = np.concatenate([v.real, v.imag], axis=1)  # [F, 2K]
    if op["doubled"]:
        rows = np.concatenate([np.concatenate([v.real, -v.imag], axis=1), np.concatenate([v.imag, v.real], axis=1)])
    return rows


def run_net(net, prm):
    """Expectation value of one network for one parameter vector."""
    leaves = {t: _leaf(net, t, prm) for t in range(net["n_leaves"])}
    total = 0.0
    for sl in range(1 << len(net["sliced"])):
        store = dict(leaves)
        for st in net["steps"]:
            if st["fused"]:
                # fused kernel: complex product written planar (Re at j*M + i, Im at + M*N)
                C = _complex(net, st["opa"], store, sl) @ _complex(net, st["opb"], store, sl).T
                store[st["out"]] = np.concatenate([C.real.T.reshape(-1), C.imag.T.reshape(-1)])
                continue
            A = _gather(net, st["opa"], store, sl)  # rows of op(A)
            B = _gather(net, st["opb"], store, sl)  # columns of B
            store[st["out"]] = (A @ B.T).reshape(-1, order="F")  # column-major result
        total += store[net["root"]][0]
    return total


def run(desc, prm):
    return np.array([run_net(net, np.asarray(prm, dtype=np.float64)) for net in desc["nets"]])


def check_arenas(net):
    """Steps run by level (inputs from lower levels only), a level's fused
    steps first and together.  Live intermediates never overlap in their
    arena (batched and unbatched separately); the output of a gathered step
    may reuse the space of its inputs, the outputs of a level's fused steps
    (which read their inputs in place, concurrently) overlap no input of the
    level and no other output."""
    T = net["tensors"]
    L = net["n_leaves"]
    steps = net["steps"]
    level_of = {}
    for st in steps:
        for t in (st["a"], st["b"]):
            if t >= L:
                assert level_of[t] < st["level"], "input from the same or a later level"
        level_of[st["out"]] = st["level"]
    keys = [(st["level"], 0 if st["fused"] else 1) for st in steps]
    assert keys == sorted(keys), "steps not ordered by level, fused first"
    live = {}

    def place(o):
        size = 2 << (T[o]["lm"] + T[o]["ln"])
        lo, hi = T[o]["arena"], T[o]["arena"] + size
        arena_max = net["batched_arena"] if T[o]["batched"] else net["unbatched_arena"]
        assert 0 <= lo and hi <= arena_max
        for t, (b, l2, h2) in live.items():
            if b == T[o]["batched"]:
                assert hi <= l2 or h2 <= lo, f"tensor {o} overlaps live tensor {t}"
        live[o] = (T[o]["batched"], lo, hi)

    i = 0
    while i < len(steps):
        j = i
        while j < len(steps) and steps[j]["fused"] and steps[j]["level"] == steps[i]["level"]:
            j += 1
        if j > i:
            for st in steps[i:j]:
                place(st["out"])
            for st in steps[i:j]:
                for t in (st["a"], st["b"]):
                    if t >= L:
                        live.pop(t)
        else:
            st = steps[i]
            for t in (st["a"], st["b"]):
                if t >= L:
                    live.pop(t)
            place(st["out"])
            j = i + 1
        i = j
    assert list(live) == [net["root"]]
