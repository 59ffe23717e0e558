"""Block-diagonal metric tensor for quantum natural gradient, on the GB300 backend.

Reference: ``Circuit.cycabc`` / ``gen_circuits`` / ``metric_tensor`` and
``cov_matrix`` (tedq/QInterpreter/circuits/circuit.py:101-203, 297-403) with
the optimizer in tedq/optimizers/quantum_natural_gradient.py.  The reference
splits the circuit into layers (a one-parameter gate selected for QNG starts a
new layer on its qubits), builds one circuit per layer -- every gate of the
earlier layers plus the diagonalising gates of the layer's generators --
measures ``probs`` of all qubits with the pytorch backend, and forms the
covariance of the generators from marginal probabilities on the host:
``g_layer = outer(f, f) * (<o_i o_j> - <o_i><o_j>)``.

Here each layer's prefix circuit is compiled once for the GB300 backend and
measures the covariance terms directly as expectation values (``<o_i>``,
``<o_i o_i>`` and ``<o_i o_j>`` as Pauli strings / matrix observables, reduced
on the device by the Walsh-Hadamard expval kernel) -- no 2^n probability
vector and no host marginals -- and every call evaluates a whole batch of
parameter vectors.  The result equals the reference's in exact arithmetic.
"""

from collections import defaultdict

import numpy as np
import torch

from .measurement import expval
from .operators import GateBase, Unitary


def layer_blocks(circuit, numarg):
    """Layering of ``circuit`` for the metric tensor (restates circuit.py
    :101-164): returns ``(layers, obs_list, factors_list, num_params)``, dicts
    keyed by layer id -- the operators of each layer, and for the layers that
    end with selected one-parameter gates the generators' observables, their
    factors and the flat indices of those parameters."""
    q_layers = [0] * circuit.num_qubits
    layers = defaultdict(list)
    obs_list = defaultdict(list)
    factors_list = defaultdict(list)
    num_params = defaultdict(list)
    numarg = set(int(n) for n in numarg)
    num = 0
    for op in circuit.operators:
        n_tp = len(op.trainable_params)
        layer = max(q_layers[q] for q in op.qubits)
        if n_tp == 1 and num in numarg:
            s, ob = op.generator
            obs_list[layer].append(ob)
            factors_list[layer].append(s)
            num_params[layer].append(num)
            layer += 1
        if n_tp > 1 and any(k in numarg for k in range(num, num + n_tp)):
            raise ValueError("quantum gate with more than one parameters can not use quantum natural gradient!")
        for q in op.qubits:
            q_layers[q] = layer
        layers[layer].append(op)
        num += n_tp
    return layers, obs_list, factors_list, num_params


def _square(ob):
    """The observable o*o (identity for Pauli observables)."""
    m = np.asarray(ob.matrix, dtype=np.complex128)
    return Unitary(m @ m, qubits=list(ob.qubits), do_queue=False)


class MetricTensor:
    """Callable block-diagonal metric tensor of ``circuit`` for the parameters
    listed in ``numarg`` (flat trainable-parameter indices).

    ``mt(*parameters)`` follows the reference's call (the circuit's flat
    parameters) and returns the ``[K, K]`` block-diagonal tensor;
    ``mt.batch(P)`` takes ``[B, n_params]`` and returns ``[B, K, K]``."""

    def __init__(self, circuit, numarg, precision="c64", **kwargs):
        from .circuit import Circuit

        self.n_params = sum(len(op.trainable_params) for op in circuit.operators)
        # flat parameter slots of every operator of the full circuit
        slots, k = {}, 0
        for op in circuit.operators:
            slots[id(op)] = list(range(k, k + len(op.trainable_params)))
            k += len(op.trainable_params)
        layers, obs_list, factors_list, num_params = layer_blocks(circuit, numarg)
        self.blocks = []
        for layer_id in sorted(obs_list):
            obs = obs_list[layer_id]
            ops = [op for i in range(layer_id + 1) for op in layers[i]]
            sel = [s for op in ops for s in slots[id(op)]]
            meas = [expval(ob, do_queue=False) for ob in obs]
            meas += [expval(_square(ob), do_queue=False) for ob in obs]
            pairs = [(i, j) for i in range(len(obs)) for j in range(i + 1, len(obs))]
            meas += [expval([obs[i], obs[j]], do_queue=False) for i, j in pairs]
            prefix = Circuit({"operators": ops, "measurements": meas, "init_state": circuit.init_state},
                             circuit.num_qubits)
            cc = prefix.compilecircuit(backend="gb300", precision=precision, requires_grad=False, **kwargs)
            self.blocks.append({"cc": cc, "sel": sel, "n": len(obs), "pairs": pairs,
                                "factors": np.asarray(factors_list[layer_id], dtype=np.float64),
                                "params": num_params[layer_id]})
        self.size = sum(b["n"] for b in self.blocks)

    def batch(self, P):
        """``[B, n_params]`` parameter vectors -> ``[B, K, K]`` metric tensors."""
        if P.dim() != 2 or P.shape[1] != self.n_params:
            raise ValueError(f"expected [B, {self.n_params}] parameters, got {tuple(P.shape)}")
        B = P.shape[0]
        out = torch.zeros((B, self.size, self.size), dtype=torch.float64)
        k0 = 0
        for b in self.blocks:
            Q = P[:, b["sel"]]
            if Q.shape[1] == 0:
                Q = P.new_zeros((B, 0))
            e = b["cc"].execute_batch(Q).detach().to(torch.float64).cpu()  # [B, measurements]
            n = b["n"]
            mean, sq = e[:, :n], e[:, n:2 * n]
            cov = torch.diag_embed(sq - mean * mean)
            for t, (i, j) in enumerate(b["pairs"]):
                c = e[:, 2 * n + t] - mean[:, i] * mean[:, j]
                cov[:, i, j] = c
                cov[:, j, i] = c
            f = torch.from_numpy(b["factors"])
            out[:, k0:k0 + n, k0:k0 + n] = cov * torch.outer(f, f)
            k0 += n
        return out

    def __call__(self, *parameters):
        flat = torch.cat([torch.as_tensor(p).reshape(-1) for p in parameters]) if parameters else torch.zeros(0)
        return self.batch(flat.reshape(1, -1).to(torch.float64))[0]


class QNG(torch.optim.Optimizer):
    """Quantum natural gradient step ``x <- x - lr * g^-1 grad`` (the update of
    tedq/optimizers/quantum_natural_gradient.py:22-99, with plain SGD
    semantics: no momentum or weight decay)."""

    def __init__(self, params, lr):
        super().__init__(params, dict(lr=lr))

    @torch.no_grad()
    def step(self, metric_tensor, closure=None):
        loss = closure() if closure is not None else None
        for group in self.param_groups:
            ps = [p for p in group["params"] if p.grad is not None]
            if not ps:
                continue
            grad = torch.cat([p.grad.reshape(-1) for p in ps]).to(torch.float64).cpu()
            g = torch.as_tensor(metric_tensor, dtype=torch.float64).cpu()
            delta = torch.linalg.solve(g, grad)
            k = 0
            for p in ps:
                n = p.numel()
                p.add_(-group["lr"] * delta[k:k + n].reshape(p.shape).to(p.dtype).to(p.device))
                k += n
        return loss
