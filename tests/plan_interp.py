"""NumPy interpreter of the compiled pass/phase schedule (test helper).

Executes the schedule exported by ``tedq_program_describe`` with exactly the
data movement the CUDA kernels perform -- tile gather through the pass's
bit map, the swizzled shared-memory image, per-phase register sets built from
``reg_off``/``tid_off``, register-level gates with control masks, dense phases,
the adjoint gradients -- but in complex128 on the CPU.  Comparing its results
with the oracle checks the scheduler, the bit and swizzle tables, the gate
lowering and the Pauli expansion of the observables without a GPU.
"""

import numpy as np

F_FIXED2, F_FIXD, F_RX, F_RY, F_RZ, F_PHASE, F_ROT = range(7)
GK_U1, GK_D1, GK_X, GK_SWAP, GK_RXT, GK_RYT, GK_PH, GK_H, GK_RXN, GK_RYN = range(10)
GR_NONE, GR_X, GR_Y, GR_Z, GR_P1 = range(5)


def swz_unit(u):
    v, f = u >> 3, 0
    while v:
        f ^= v & 7
        v >>= 3
    return u ^ f


def _factor(F, fixed, prm):
    def val(j):
        return prm[F["slot"][j]] if F["slot"][j] >= 0 else F["val"][j]
    op = F["op"]
    if op == F_FIXED2:
        return np.array(fixed[F["fix"]:F["fix"] + 4]).reshape(2, 2)
    if op == F_FIXD:
        return np.diag(fixed[F["fix"]:F["fix"] + 2])
    th = val(0)
    c, s = np.cos(th / 2), np.sin(th / 2)
    if op == F_RX:
        return np.array([[c, -1j * s], [-1j * s, c]])
    if op == F_RY:
        return np.array([[c, -s], [s, c]], dtype=complex)
    if op == F_RZ:
        return np.diag([c - 1j * s, c + 1j * s])
    if op == F_PHASE:
        return np.diag([1, np.exp(1j * th)])
    raise ValueError(op)


def _normalised(M, rx):
    """Normalised rotation (GK_RXN / GK_RYN): the gate divided by the larger
    of |c|, |s| with its global phase dropped; returns (matrix, scale)."""
    c = M[0, 0].real
    s = -M[0, 1].imag if rx else -M[0, 1].real
    if abs(c) >= abs(s):
        t = s / c
        N = np.array([[1, -1j * t], [-1j * t, 1]]) if rx else np.array([[1, -t], [t, 1]], dtype=complex)
        return N, abs(c)
    u = c / s
    N = np.array([[1j * u, 1], [1, 1j * u]]) if rx else np.array([[u, -1], [1, u]], dtype=complex)
    return N, abs(s)


def _mats(P, prm):
    fixed = [complex(a, b) for a, b in P["fixed"]]
    out, sig = [], []
    for md in P["mats"]:
        M = np.eye(2, dtype=complex)
        for F in md["factors"]:
            M = _factor(F, fixed, prm) @ M
        if md["dagger"]:
            M = M.conj().T
        sg = 1.0
        if md["diag"] == 2:  # global phase dropped: diag(1, d1 / d0)
            M = np.diag([1.0, M[1, 1] * np.conj(M[0, 0])])
        elif md["diag"] >= 3:
            M, sg = _normalised(M, md["diag"] == 3)
        out.append(M)
        sig.append(sg)
    return out, fixed, sig


def _apply(a, r, M):
    """Apply register gate r to a[:, 0:2^R] in place."""
    k0, cm, kind = r["k0"], r["cmask"], r["kind"]
    NR = a.shape[1]
    if kind == GK_SWAP:
        b0, b1 = 1 << k0, 1 << r["k1"]
        for tgt, c in ((r["k1"], cm | b0), (k0, cm | b1), (r["k1"], cm | b0)):
            _apply(a, {"kind": GK_X, "k0": tgt, "cmask": c}, None)
        return
    if kind == GK_RXT:
        c, sn = M[0, 0].real, -M[0, 1].imag
        M = np.array([[c, -1j * sn], [-1j * sn, c]])
        kind = GK_U1
    elif kind == GK_RYT:
        c, sn = M[0, 0].real, -M[0, 1].real
        M = np.array([[c, -sn], [sn, c]], dtype=complex)
        kind = GK_U1
    elif kind == GK_PH:
        M = np.diag([1.0, M[1, 1]])
        kind = GK_D1
    elif kind == GK_H:
        M = np.array([[1.0, 1.0], [1.0, -1.0]], dtype=complex) / np.sqrt(2.0)
        kind = GK_U1
    elif kind in (GK_RXN, GK_RYN):
        kind = GK_U1
    for i in range(NR):
        if kind == GK_D1:
            if (i & cm) == cm:
                a[:, i] *= M[1, 1] if (i >> k0) & 1 else M[0, 0]
            continue
        if i & (1 << k0) or (i & cm) != cm:
            continue
        j = i | (1 << k0)
        x0, x1 = a[:, i].copy(), a[:, j].copy()
        if kind == GK_X:
            a[:, i], a[:, j] = x1, x0
        else:
            a[:, i] = M[0, 0] * x0 + M[0, 1] * x1
            a[:, j] = M[1, 0] * x0 + M[1, 1] * x1


def _grad(a, l, r):
    k0, cm, g = r["k0"], r["cmask"], r["grad"]
    acc = 0.0
    for i in range(a.shape[1]):
        if i & (1 << k0) or (i & cm) != cm:
            continue
        j = i | (1 << k0)
        p0, p1, l0, l1 = a[:, i], a[:, j], l[:, i], l[:, j]
        if g == GR_X:
            acc += np.sum((np.conj(l0) * p1 + np.conj(l1) * p0).imag)
        elif g == GR_Y:
            acc += np.sum((np.conj(l1) * p0).real - (np.conj(l0) * p1).real)
        elif g == GR_Z:
            acc += np.sum((np.conj(l0) * p0 - np.conj(l1) * p1).imag)
        else:
            acc += np.sum((np.conj(l1) * p1).imag)
    return acc * r["coef"]


def _dense(tile_phys, P, ph, fixed, m, e):
    k, d = ph["dk"], 1 << ph["dk"]
    pos = ph["dpos"][:k]
    Mx = np.array(fixed[ph["dfix"]:ph["dfix"] + d * d]).reshape(d, d)
    if ph["dagger"]:
        Mx = Mx.conj().T
    dmask = sum(1 << p for p in pos)
    free = [p for p in range(m) if not (dmask >> p) & 1]
    for grp in range(1 << (m - k)):
        base = sum(((grp >> i) & 1) << p for i, p in enumerate(free))
        if (base & ph["dcmask"]) != ph["dcmask"]:
            continue
        addr = []
        for r in range(d):
            t = base
            for i in range(k):
                if (r >> (k - 1 - i)) & 1:
                    t |= 1 << pos[i]
            addr.append((swz_unit(t >> e) << e) | (t & ((1 << e) - 1)))
        v = tile_phys[addr]
        tile_phys[addr] = Mx @ v


def _tile_index(P, tile):
    """Global amplitude index of every tile offset t (vector over t)."""
    m, c = P["m"], P["c"]
    base = 0
    for k, b in enumerate(P["outer"]):
        if (tile >> k) & 1:
            base |= 1 << b
    t = np.arange(1 << m)
    g = base | (t & ((1 << c) - 1))
    h = t >> c
    for k, b in enumerate(P["hi"]):
        g = g | (((h >> k) & 1) << b)
    return g


def run_pass(P, psi, prm, lam=None, grads=None):
    m, e, R = P["m"], P["e"], P["R"]
    mats, fixed, sig = _mats(P, prm)
    n_outer = len(P["outer"])
    T = 1 << (m - R)
    phys = np.array([(swz_unit(t >> e) << e) | (t & ((1 << e) - 1)) for t in range(1 << m)])
    zero_outer = P.get("zero_outer", 0)
    for tile in range(1 << n_outer):
        g = _tile_index(P, tile)
        if zero_outer and (int(g[0]) & zero_outer):
            # the device skips this tile: it must be (and stays) all zero
            assert not np.any(psi[g]), "a tile the kernels skip holds non-zero amplitudes"
            continue
        tp = np.zeros(1 << m, dtype=complex)
        tp[phys] = psi[g]
        tl = None
        if lam is not None:
            tl = np.zeros(1 << m, dtype=complex)
            tl[phys] = lam[g]
        kap = 1.0  # states carry 1 / (product of normalised-rotation scales so far)
        for f, ph in enumerate(P["phases"]):
            if ph["type"] == 1:
                _dense(tp, P, ph, fixed, m, e)
                if tl is not None:
                    _dense(tl, P, ph, fixed, m, e)
                continue
            tids = np.arange(T)
            bu = np.zeros(T, dtype=np.int64)
            for b, off in enumerate(ph["tid_off"]):
                bu ^= np.where((tids >> b) & 1, off, 0)
            NR = 1 << R
            addr = np.zeros((T, NR), dtype=np.int64)
            for j in range(NR):
                unit = bu ^ ph["reg_off"][j >> e]
                addr[:, j] = (unit << e) | (j & ((1 << e) - 1))
            a = tp[addr]
            l = tl[addr] if tl is not None else None
            for r in ph["gates"]:
                M = mats[r["mat"]] if r["kind"] not in (GK_X, GK_SWAP, GK_H) else None
                if l is not None and r["grad"] != GR_NONE:
                    grads[r["slot"]] += _grad(a, l, r) * kap * kap
                _apply(a, r, M)
                if l is not None:
                    _apply(l, r, M)
                if r["kind"] in (GK_RXN, GK_RYN):
                    kap *= sig[r["mat"]]
            if f == P.get("norm_phase", -1):
                a *= kap
                if l is not None:
                    l *= kap
                kap = 1.0
            tp[addr] = a
            if tl is not None:
                tl[addr] = l
        psi[g] = tp[phys]
        if lam is not None:
            lam[g] = tl[phys]


def pauli_apply(psi, x, z):
    """(P_h psi)(w) = (-i)^ny (-1)^{popcount(z & w)} psi(w ^ x)."""
    w = np.arange(psi.size)
    ny = bin(x & z).count("1")
    par = np.array([bin(v).count("1") & 1 for v in (w & z)])
    return ((-1j) ** ny) * np.where(par, -1, 1) * psi[w ^ x]


def forward(desc, prm, init=None):
    """From |0...0> the passes skip the tiles their zero_outer masks name (as
    the kernels do, after clearing the state); a given initial state runs
    every tile (the launcher clears the masks)."""
    ns = desc["state_qubits"]
    psi = np.zeros(1 << ns, dtype=complex)
    if init is None:
        psi[0] = 1
    else:
        pad = ns - desc["n"]
        psi[::1 << pad] = init
    for P in desc["passes"]:
        run_pass(P if init is None else dict(P, zero_outer=0), psi, prm)
    return psi


def outputs(desc, psi):
    out = np.zeros(desc["n_real"])
    vals = [float(np.real(np.vdot(psi, pauli_apply(psi, x, z)))) for x, z in desc["terms"]]
    for k, s, c in desc["out_terms"]:
        out[k] += c * vals[s]
    pad = desc["state_qubits"] - desc["n"]
    for pr in desc["probs"]:
        p = np.abs(psi) ** 2
        w = np.arange(psi.size)
        nb = len(pr["bits"])
        b = np.zeros(psi.size, dtype=np.int64)
        for bit in pr["bits"]:
            b = (b << 1) | ((w >> bit) & 1)
        keep = (w & ((1 << pad) - 1)) == 0
        out[pr["offset"]:pr["offset"] + (1 << nb)] = np.bincount(b[keep], weights=p[keep], minlength=1 << nb)
    return out


def adjoint(desc_bwd, prm, psi, dy_real, dy_state=None):
    lam = np.zeros_like(psi)
    w = np.zeros(len(desc_bwd["terms"]))
    for k, s, c in desc_bwd["out_terms"]:
        w[s] += c * dy_real[k]
    for (x, z), ws in zip(desc_bwd["terms"], w):
        lam += ws * pauli_apply(psi, x, z)
    idx = np.arange(psi.size)
    pad = desc_bwd["state_qubits"] - desc_bwd["n"]
    for pr in desc_bwd["probs"]:
        b = np.zeros(psi.size, dtype=np.int64)
        for bit in pr["bits"]:
            b = (b << 1) | ((idx >> bit) & 1)
        lam += dy_real[pr["offset"] + b] * psi * ((idx & ((1 << pad) - 1)) == 0)
    if dy_state is not None:
        lam += 0.5 * dy_state
    grads = np.zeros(desc_bwd["n_params"])
    for P in desc_bwd["passes"]:
        run_pass(P, psi, prm, lam, grads)
    return grads
