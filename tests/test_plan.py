"""CPU checks of the compiled schedule (no GPU): the native compile step runs
on the host; its exported pass/phase plan is executed by ``plan_interp`` in
complex128 and compared with the reference's golden outputs and gradients."""

import numpy as np
import pytest
import torch

import plan_interp
from conftest import load_cases

qai = pytest.importorskip("tedq_gb300")

CASES = load_cases()


def _arr(v):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 2 and a.shape[1] == 2:
        return a[:, 0] + 1j * a[:, 1]
    return a


def _compile(case, precision, fuse=True):
    circ = qai.Circuit.from_spec(case)
    return circ.compilecircuit(backend="gb300", precision=precision, fuse=fuse)


def _assemble(case, desc, out, psi):
    pad = desc["state_qubits"] - desc["n"]
    res = []
    k = 0
    for m in case["meas"]:
        if m["kind"] == "expval":
            res.append(np.array([out[k]]))
            k += 1
        elif m["kind"] == "probs":
            q = case["n"] if m["qubits"] is None else len(set(m["qubits"]))
            res.append(out[k:k + 2 ** q])
            k += 2 ** q
        else:
            res.append(psi[:: 1 << pad])
    return np.concatenate(res)


def _init(case):
    if case.get("init_state") is None:
        return None
    return _arr(case["init_state"])


@pytest.mark.parametrize("precision", ["c64", "c128"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_plan_forward_matches_reference(case, precision):
    cc = _compile(case, precision)
    desc = cc.describe()
    prm = np.asarray(case["params"], dtype=np.float64)
    psi = plan_interp.forward(desc, prm, _init(case))
    got = _assemble(case, desc, plan_interp.outputs(desc, psi), psi)
    np.testing.assert_allclose(got, _arr(case["out_c128"]), atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("case", [c for c in CASES if c["params"]], ids=[c["name"] for c in CASES if c["params"]])
def test_plan_adjoint_matches_reference(case):
    cc = _compile(case, "c128")
    fwd, bwd = cc.describe(), cc.describe(adjoint=True)
    prm = np.asarray(case["params"], dtype=np.float64)
    psi = plan_interp.forward(fwd, prm, _init(case))
    dy = np.asarray(case["dy"], dtype=np.float64)
    # split dy into the real outputs and the state outputs, in measurement order
    dy_real = np.zeros(fwd["n_real"])
    dy_state = None
    per = int(np.prod(case["shape"][1:])) if len(case["shape"]) > 1 else 1
    pad = fwd["state_qubits"] - fwd["n"]
    k = 0
    for i, m in enumerate(case["meas"]):
        chunk = dy[i * per:(i + 1) * per]
        if m["kind"] == "state":
            full = np.zeros(psi.size, dtype=complex)
            full[:: 1 << pad] = chunk
            dy_state = full if dy_state is None else dy_state + full
        else:
            dy_real[k:k + per] = chunk
            k += per
    g = plan_interp.adjoint(bwd, prm, psi.copy(), dy_real, dy_state)
    np.testing.assert_allclose(g, case["grad_backprop_c128"], atol=1e-10, rtol=1e-9)


def _same_up_to_phase(a, b, atol):
    ov = np.vdot(b, a)
    np.testing.assert_allclose(abs(ov), 1.0, atol=atol)
    np.testing.assert_allclose(a, b * (ov / abs(ov)), atol=atol)


def test_plan_unfused_matches_fused():
    case = next(c for c in CASES if c["name"] == "all_gates_n4")
    prm = np.asarray(case["params"], dtype=np.float64)
    a = plan_interp.forward(_compile(case, "c64", fuse=True).describe(), prm)
    b = plan_interp.forward(_compile(case, "c64", fuse=False).describe(), prm)
    # without a state output, diagonal gates may drop their global phase
    _same_up_to_phase(a, b, 1e-12)


def _phase_case():
    return {"name": "rz_phase", "n": 3, "init_state": None,
            "gates": [{"name": "RY", "qubits": [0], "params": [0.3], "trainable": [0]},
                      {"name": "RZ", "qubits": [0], "params": [0.7], "trainable": [0]},
                      {"name": "RZ", "qubits": [1], "params": [1.1], "trainable": [0]},
                      {"name": "T", "qubits": [2], "params": [], "trainable": []},
                      {"name": "CRZ", "qubits": [0, 2], "params": [0.4], "trainable": [0]},
                      {"name": "PhaseShift", "qubits": [1], "params": [0.9], "trainable": [0]}],
            "meas": [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [0]}]}],
            "params": [0.3, 0.7, 1.1, 0.4, 0.9]}


def test_plan_phase_dropping_and_exact_phase():
    """Uncontrolled diagonal gates drop their global phase only without a
    state output; exact_phase=1 (and any state measurement) keeps it."""
    case = _phase_case()
    circ = qai.Circuit.from_spec(case)
    free = circ.compilecircuit(backend="gb300", precision="c128").describe()
    exact = circ.compilecircuit(backend="gb300", precision="c128", exact_phase=True).describe()
    kinds = lambda d: sorted(md["diag"] for P in d["passes"] for md in P["mats"])
    assert 2 in kinds(free) and 2 not in kinds(exact)
    prm = np.asarray(case["params"], dtype=np.float64)
    a = plan_interp.forward(free, prm)
    b = plan_interp.forward(exact, prm)
    _same_up_to_phase(a, b, 1e-12)
    # the exact program's state is the reference state, phase included
    import oracle
    spec = dict(case, meas=[{"kind": "state"}])
    want = oracle.run(spec, torch.tensor(prm), torch.complex128).numpy().reshape(-1)
    pad = exact["state_qubits"] - exact["n"]
    np.testing.assert_allclose(b[:: 1 << pad], want, atol=1e-12)
    # a state measurement alone also keeps the phase
    st = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", precision="c128").describe()
    assert 2 not in kinds(st)
    # the adjoint sweep always drops it; its gradients still match the reference
    g = plan_interp.adjoint(circ.compilecircuit(backend="gb300", precision="c128").describe(adjoint=True), prm,
                            a.copy(), np.ones(free["n_real"]), None)
    _, want_g = oracle.value_and_grad(case, torch.tensor(prm), [1.0], torch.complex128)
    np.testing.assert_allclose(g, want_g.numpy(), atol=1e-10)





def _hea_spec(n, layers, seed):
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
    meas.append({"kind": "expval", "list": True, "obs": [{"name": "PauliZ", "qubits": [0]},
                                                        {"name": "PauliZ", "qubits": [1]}]})
    return {"n": n, "gates": gates, "meas": meas, "init_state": None}


@pytest.mark.parametrize("n,tile", [(14, 0), (15, 11), (16, 10)])
def test_plan_multi_pass_against_oracle(n, tile):
    """States larger than one tile: several passes with non-trivial outer bits."""
    import oracle
    spec = _hea_spec(n, 2, seed=n)
    circ = qai.Circuit.from_spec(spec)
    cc = circ.compilecircuit(backend="gb300", precision="c128", tile_qubits=tile)
    desc = cc.describe()
    assert len(desc["passes"]) >= 2
    prm = np.array([g["params"][0] for g in spec["gates"] if g["trainable"]])
    psi = plan_interp.forward(desc, prm)
    want = oracle.run(spec, torch.tensor(prm, dtype=torch.float64), torch.complex128).numpy()
    np.testing.assert_allclose(plan_interp.outputs(desc, psi), want, atol=1e-12)
    dy = np.linspace(-1, 1, len(want))
    g = plan_interp.adjoint(cc.describe(adjoint=True), prm, psi.copy(), dy)
    _, want_g = oracle.value_and_grad(spec, prm, dy, torch.complex128)
    np.testing.assert_allclose(g, want_g.numpy(), atol=1e-11)


@pytest.mark.parametrize("n,adjoint", [(12, False), (16, False), (16, True), (20, True)])
def test_staging_tables_match_tile_map(n, adjoint):
    """gtid/gk/stid/sk reproduce the tile gather and the swizzle for every unit."""
    spec = _hea_spec(n, 2, seed=1)
    desc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300").describe(adjoint=adjoint)
    for P in desc["passes"]:
        m, e, R = P["m"], P["e"], P["R"]
        T, NU = 1 << (m - R), 1 << (R - e)
        g_direct = plan_interp._tile_index(P, 0)
        for tid in range(T):
            g_t, s_t = 0, 0
            for b in range(m - R):
                if (tid >> b) & 1:
                    g_t |= P["gtid"][b]
                    s_t ^= P["stid"][b]
            for k in range(NU):
                u = tid + k * T
                assert (g_t | P["gk"][k]) == g_direct[u << e]
                assert (s_t ^ P["sk"][k]) == plan_interp.swz_unit(u)


@pytest.mark.parametrize("norm", ["0", "f", "b", "fbu"])
def test_plan_register_gate_forms(monkeypatch, norm):
    """Every choice of register-gate forms (TEDQ_GB300_NORMALISE) reproduces
    the reference's outputs and gradients on the golden cases."""
    monkeypatch.setenv("TEDQ_GB300_NORMALISE", norm)
    for case in [c for c in CASES if c["params"]]:
        cc = _compile(case, "c128", fuse=(norm != "f"))
        fwd, bwd = cc.describe(), cc.describe(adjoint=True)
        prm = np.asarray(case["params"], dtype=np.float64)
        psi = plan_interp.forward(fwd, prm, _init(case))
        got = _assemble(case, fwd, plan_interp.outputs(fwd, psi), psi)
        if any(m["kind"] == "state" for m in case["meas"]):
            continue
        np.testing.assert_allclose(got, _arr(case["out_c128"]), atol=1e-12, rtol=1e-12)
        dy = np.asarray(case["dy"], dtype=np.float64)
        g = plan_interp.adjoint(bwd, prm, psi.copy(), dy[:fwd["n_real"]], None)
        np.testing.assert_allclose(g, case["grad_backprop_c128"], atol=1e-10, rtol=1e-9)


def _warp_units(ph, e, R, warp):
    units = set()
    for lane in range(32):
        tid = warp * 32 + lane
        bu = 0
        for b, off in enumerate(ph["tid_off"]):
            if (tid >> b) & 1:
                bu ^= off
        for j in range(1 << (R - e)):
            units.add(bu ^ ph["reg_off"][j])
    return units


def _check_warp_local(desc):
    marked = total = 0
    for P in desc["passes"]:
        e, R = P["e"], P["R"]
        prev = None
        for ph in P["phases"]:
            if ph["type"] != 0:
                assert not ph.get("wlocal")
                prev = None
                continue
            if prev is not None:
                total += 1
            if ph["wlocal"]:
                assert prev is not None
                marked += 1
                for w in range(1 << (len(ph["tid_off"]) - 5)):
                    assert _warp_units(prev, e, R, w) == _warp_units(ph, e, R, w)
            prev = ph
    return marked, total


@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_plan_warp_local_transitions_golden_cases(precision):
    """Warp-local marks stay exact on every golden case (dense phases,
    controlled and three-qubit gates, small padded states), both sweeps."""
    for case in CASES:
        cc = _compile(case, precision)
        for adjoint in (False, True):
            if adjoint and not case["params"]:
                continue
            _check_warp_local(cc.describe(adjoint=adjoint))


@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("n,layers", [(14, 3), (20, 10)])
def test_plan_warp_local_transitions(n, layers, adjoint):
    """A register phase marked warp-local touches, in every warp, exactly the
    shared-memory units the warp touched in the previous register phase (the
    kernels then separate the two phases with __syncwarp only)."""
    spec = _hea_spec(n, layers, seed=n)
    desc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300").describe(adjoint=adjoint)
    marked = total = 0
    for P in desc["passes"]:
        e, R = P["e"], P["R"]
        nwarps = 1 << max(0, len(P["phases"][0].get("tid_off", [])) - 5) if P["phases"] else 1
        prev = None
        for ph in P["phases"]:
            if ph["type"] != 0:
                assert not ph.get("wlocal")
                prev = None
                continue
            if prev is not None:
                total += 1
            if ph["wlocal"]:
                assert prev is not None
                marked += 1
                for w in range(1 << (len(ph["tid_off"]) - 5)):
                    assert _warp_units(prev, e, R, w) == _warp_units(ph, e, R, w)
            prev = ph
    assert total == 0 or marked > 0


def _vqc20_spec():
    """The 20-qubit, 10-layer VQC of the benchmark (RX RY RZ per qubit, CNOT ladder)."""
    rng = np.random.default_rng(0)
    gates = []
    for _ in range(10):
        for q in range(20):
            for name in ("RX", "RY", "RZ"):
                gates.append({"name": name, "qubits": [q], "params": [float(rng.uniform(0, 2 * np.pi))],
                              "trainable": [0]})
        for q in range(19):
            gates.append({"name": "CNOT", "qubits": [q, q + 1], "params": [], "trainable": []})
    meas = [{"kind": "expval", "list": False, "obs": [{"name": "PauliZ", "qubits": [q]}]} for q in range(20)]
    return {"n": 20, "gates": gates, "meas": meas, "init_state": None}


@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_pass_launch_variants(precision):
    """Launch variant of every specialised pass (describe's 'pipelined',
    'groups', 'cta_smem'): the VQC's passes (short or rotation-heavy) are
    pipelined with two thread groups in complex64; the MBL chain's long passes
    of Hadamard, CNOT and phase gates run one tile per CTA; a small circuit's
    whole-state tile runs one tile per CTA; every CTA fits in 227 KB of
    shared memory."""
    from tedq_gb300.templates import mbl_spec
    cases = {"vqc": _vqc20_spec(), "mbl": mbl_spec(24, 3, seed=0), "hea8": _hea_spec(8, 2, seed=1)}
    for name, spec in cases.items():
        cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", precision=precision, jit=-1)
        for adjoint in (False, True):
            for P in cc.describe(adjoint=adjoint)["passes"]:
                assert P["cta_smem"] <= 227 * 1024
                n_gates = sum(len(ph.get("gates", [])) for ph in P["phases"])
                if name == "hea8":
                    assert P["pipelined"] == 0
                if P["pipelined"]:
                    assert P["groups"] == 2
                if name == "vqc" and precision == "c64":
                    assert P["pipelined"] == 1
                if name == "mbl" and n_gates > 64:
                    assert P["pipelined"] == 0


@pytest.mark.parametrize("G", [1, 2])
def test_tile_slot_protocol(G):
    """The pipelined kernel's slot schedule, restated: tile k of a CTA's range
    belongs to group k % G and lives in slot k % (G + 1); tile j < G + 1 is
    fetched at start by group (j + G - 1) % G, every later tile k + G + 1 by
    the group that finished tile k, into the slot it freed.  Under every
    interleaving of the groups each tile is fetched exactly once, into a free
    slot, before its group waits for it, and no group waits for a tile that
    nobody will fetch (no deadlock)."""
    import random
    for cnt in range(0, 24):
        for seed in range(12):
            rnd = random.Random(seed)
            fetched, slot_of = set(), {}
            for j in range(min(G + 1, cnt)):
                assert (j + G - 1) % G in range(G)
                fetched.add(j)
                slot_of[j % (G + 1)] = j
            k = [g - G for g in range(G)]
            state = ["next"] * G
            done, steps = set(), 0
            while any(st != "exit" for st in state):
                steps += 1
                assert steps < 10000, "deadlock"
                g = rnd.randrange(G)
                if state[g] == "exit":
                    continue
                if state[g] == "next":
                    nk = k[g] + G
                    if nk >= cnt:
                        state[g] = "exit"
                    elif nk in fetched:
                        k[g] = nk
                        state[g] = "work"
                    continue
                t = k[g]
                assert slot_of[t % (G + 1)] == t
                done.add(t)
                del slot_of[t % (G + 1)]
                nxt = t + G + 1
                if nxt < cnt:
                    assert nxt not in fetched and (nxt + G - 1) % G == g
                    fetched.add(nxt)
                    slot_of[nxt % (G + 1)] = nxt
                state[g] = "next"
            assert done == set(range(cnt))


def test_zero_tile_masks():
    """Forward sweeps from |0...0> skip all-zero tiles: a pass's zero_outer
    mask holds exactly its outer bits that no earlier forward pass had among
    its tile bits (the first pass: all its outer bits); adjoint passes have
    none."""
    spec = _vqc20_spec()
    cc = qai.Circuit.from_spec(spec).compilecircuit(backend="gb300", jit=-1)
    touched = 0
    for P in cc.describe()["passes"]:
        tile = ((1 << P["c"]) - 1) | sum(1 << b for b in P["hi"])
        outer = sum(1 << b for b in P["outer"])
        assert P["zero_outer"] == outer & ~touched
        touched |= tile
    assert cc.describe()["passes"][0]["zero_outer"] == sum(1 << b for b in cc.describe()["passes"][0]["outer"])
    assert all(P["zero_outer"] == 0 for P in cc.describe(adjoint=True)["passes"])
