"""Test helpers: golden fixtures, op conversion, and a numpy interpreter of
host-built plans (a checker for the fuser; never used by the engine)."""

from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from pyquafu_gb300 import ir

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def op_from_json(d) -> ir.Op:
    m = None
    if "matrix" in d:
        m = np.array(d["matrix"][0]) + 1j * np.array(d["matrix"][1])
    body = [op_from_json(b) for b in d.get("body", [])]
    return ir.Op(d["name"], d["kind"], d["qubits"], d["ncontrols"], d["params"], matrix=m, slot=d.get("slot", -1),
                 qbits=d.get("qbits", ()), cbits=d.get("cbits", ()), condition=d.get("condition", 0), body=body)


def load_golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    states = dict(np.load(os.path.join(GOLDEN, "golden_states.npz")))
    return meta, states


# ------------------------- engine record layouts -------------------------

PASS_DT = np.dtype([("type", "<i4"), ("T", "<i4"), ("L", "<i4"), ("H", "<i4"), ("step_begin", "<i4"),
                    ("step_count", "<i4"), ("op_begin", "<i4"), ("op_count", "<i4"), ("probe_base", "<i4"),
                    ("nprobe", "<i4"), ("tq", "u1", (16,))])
STEP_DT = np.dtype([("type", "<i4"), ("op_begin", "<i4"), ("op_count", "<i4"), ("rpos", "u1", (8,)),
                    ("tpos", "u1", (16,)), ("tglob", "u1", (16,)), ("rsw", "<u2", (8,)), ("tsw", "<u2", (16,))])
KOP_DT = np.dtype([("kind", "u1"), ("flags", "u1"), ("special", "u1"), ("k", "u1"), ("t0", "u1"), ("t1", "u1"),
                   ("probe", "<u2"), ("creg", "<u4"), ("preg", "<u4"), ("cthr", "<u8"),
                   ("pthr", "<u8"), ("coef", "<u4"), ("tk", "u1", (6,)), ("pad2", "u1", (2,)), ("xreg", "<u4")],
                  align=True)
assert PASS_DT.itemsize == 56 and STEP_DT.itemsize == 100 and KOP_DT.itemsize == 48

K_DENSE, K_REAL, K_RX, K_DIAG, K_X, K_Y, K_SWAP, K_DENSE2, K_DENSEK, K_PROBE, K_HAD, K_DIAGR = range(1, 13)
PASS_TILE, PASS_SMALL, PASS_GLOBALOP = 0, 1, 2
STEP_ROUND, STEP_SMEM = 0, 1


def host_plan(n, ops, precision=0, T=0, R=0, adjoint=False, batched=False):
    from pyquafu_gb300 import _native as nat

    lib = nat.load()
    arr, pool = ir.pack(ops)
    h = ctypes.c_void_p()
    if batched:
        nat.check(lib.qfvm_plan_host_build_batched(n, precision, nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, int(adjoint),
                                                   ctypes.byref(h)), "host batched plan")
    elif adjoint:
        nat.check(lib.qfvm_plan_host_build_adjoint(n, precision, nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, ctypes.byref(h)),
                  "host adjoint plan")
    else:
        nat.check(lib.qfvm_plan_host_build(n, precision, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                                           pool.size, T, R, ctypes.byref(h)), "host plan")
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(lib.qfvm_plan_host_counts(h, counts, shape))
    passes = np.zeros(counts[0], PASS_DT)
    steps = np.zeros(max(counts[1], 1), STEP_DT)
    kops = np.zeros(max(counts[2], 1), KOP_DT)
    coef = np.zeros(max(counts[3], 1), np.float64)
    nat.check(lib.qfvm_plan_host_copy(h, nat.vptr(passes), nat.vptr(steps), nat.vptr(kops), nat.dptr(coef)))
    nprobe = int(sum(int(p["nprobe"]) for p in passes))
    slots = np.zeros(max(nprobe, 1), dtype=np.int32)
    if nprobe:
        nat.check(lib.qfvm_plan_host_probe_slots(h, nat.i32ptr(slots)))
    nb = ctypes.c_int64()
    nat.check(lib.qfvm_plan_host_binds(h, ctypes.byref(nb), None))
    binds = np.zeros((max(nb.value, 1), 4), dtype=np.int32)
    nat.check(lib.qfvm_plan_host_binds(h, ctypes.byref(nb), nat.i32ptr(binds)))
    lib.qfvm_plan_destroy(h)
    return {"passes": passes, "steps": steps[: counts[1]], "ops": kops[: counts[2]], "coef": coef,
            "T": shape[0], "R": shape[1], "L": shape[2], "probe_slots": slots[:nprobe], "binds": binds[: nb.value],
            "elem_bytes": 8 if precision == 1 else 16}


def tile_off(s, elem_bytes):
    """The tile passes' shared-memory layout: element offset of tile index s
    (runs of 32 amplitudes contiguous, each run padded by 16 bytes times
    r + r/8 + r/64)."""
    u = 16 // elem_bytes
    return s + u * ((s >> 5) + (s >> 8) + (s >> 11))


def slot_bit(p, elem_bytes, access):
    """Bit of the 128-byte wavefront slot (of `access` bytes) that tile
    position p selects, or -1."""
    b = tile_off(1 << p, elem_bytes) * elem_bytes
    if b % access:
        return -1
    c = (b // access) % (128 // access)
    return c.bit_length() - 1 if c and not c & (c - 1) else -1


def _bits(mask):
    return [q for q in range(64) if (int(mask) >> q) & 1]


def apply_global(psi, kind, t, cmask, pmask, flags, special, coef, off, tk=()):
    """Apply one op given in global qubit terms to psi (in place)."""
    N = psi.size
    idx = np.arange(N, dtype=np.int64)
    ctrl = (idx & cmask) == cmask
    if kind == K_DIAG:
        par = np.zeros(N, dtype=np.int64)
        for q in _bits(pmask):
            par ^= (idx >> q) & 1
        if flags & 2:
            d1 = {1: -1.0, 2: 1j, 3: -1j}[special]
            d0 = 1.0
        else:
            d0 = coef[off] + 1j * coef[off + 1]
            d1 = coef[off + 2] + 1j * coef[off + 3]
        fac = np.where(par == 1, d1, d0)
        psi[:] = np.where(ctrl, psi * fac, psi)
        return
    if kind in (K_SWAP, K_DENSE2):
        t0, t1 = t
        sel = ctrl & (((idx >> t0) & 1) == 0) & (((idx >> t1) & 1) == 0)
        i = idx[sel]
        v = [psi[i], psi[i | (1 << t0)], psi[i | (1 << t1)], psi[i | (1 << t0) | (1 << t1)]]
        if kind == K_SWAP:
            out = [v[0], v[2], v[1], v[3]]
        else:
            m = (coef[off:off + 32:2] + 1j * coef[off + 1:off + 32:2]).reshape(4, 4)
            out = [sum(m[r, c] * v[c] for c in range(4)) for r in range(4)]
        for r, j in enumerate([i, i | (1 << t0), i | (1 << t1), i | (1 << t0) | (1 << t1)]):
            psi[j] = out[r]
        return
    if kind == K_DENSEK:
        k = len(tk)
        sel = ctrl.copy()
        for q in tk:
            sel &= ((idx >> q) & 1) == 0
        i = idx[sel]
        dim = 1 << k
        m = (coef[off:off + 2 * dim * dim:2] + 1j * coef[off + 1:off + 2 * dim * dim:2]).reshape(dim, dim)
        cols = []
        for c in range(dim):
            j = i.copy()
            for b, q in enumerate(tk):
                if (c >> b) & 1:
                    j |= 1 << q
            cols.append(j)
        vals = np.stack([psi[j] for j in cols])
        out = m @ vals
        for c in range(dim):
            psi[cols[c]] = out[c]
        return
    sel = ctrl & (((idx >> t) & 1) == 0)
    i0 = idx[sel]
    i1 = i0 | (1 << t)
    a, b = psi[i0].copy(), psi[i1].copy()
    if kind == K_X:
        na, nb = b, a
    elif kind == K_Y:
        na, nb = -1j * b, 1j * a
    elif kind == K_HAD:
        na, nb = a + b, a - b
    elif kind == K_REAL:
        m = coef[off:off + 4]
        na, nb = m[0] * a + m[1] * b, m[2] * a + m[3] * b
    elif kind == K_RX:
        c, s = coef[off], coef[off + 1]
        na, nb = c * a - 1j * s * b, -1j * s * a + c * b
    elif kind == K_DENSE:
        m = coef[off:off + 8:2] + 1j * coef[off + 1:off + 8:2]
        na, nb = m[0] * a + m[1] * b, m[2] * a + m[3] * b
    else:
        raise ValueError(kind)
    psi[i0], psi[i1] = na, nb


def probe_value(psi, lam, xmask, zmask, cmask, ny, scale):
    """Im <lam| Q |psi> with (Q psi)[i] = scale i^ny (-1)^popc((i^x)&z) psi[i^x] on controls."""
    idx = np.arange(psi.size, dtype=np.int64)
    ix = idx ^ xmask
    par = np.zeros(psi.size, dtype=np.int64)
    for q in _bits(zmask):
        par ^= (ix >> q) & 1
    w = psi[ix] * np.where(par == 1, -1.0, 1.0) * (1j ** ny)
    ok = (idx & cmask) == cmask
    return float(scale * np.sum(np.where(ok, np.conj(lam) * w, 0)).imag)


def kop_targets(o):
    """Targets and parity mask of a whole-state op record: a dense gate on
    more than 6 targets carries its ascending targets as the mask pthr."""
    if int(o["kind"]) == K_DENSEK and int(o["k"]) > 6:
        return [q for q in range(64) if (int(o["pthr"]) >> q) & 1], 0
    return [int(x) for x in o["tk"][: o["k"]]], int(o["pthr"])


def diagr_codes(o):
    """3-bit entry codes of a K_DIAGR op: entries 0..20 in cthr, 21..31 in pthr."""
    return int(o["cthr"]) | (int(o["pthr"]) << 63)


def apply_diagr(psi, g_of_reg, coef, off, codes):
    """A merged register-round diagonal: amplitude i *= d[j], j the register
    index of i (bit b of j = bit g_of_reg[b] of i); entries coded exactly
    1, -1, i, -i (3-bit codes) must equal their coefficients."""
    idx = np.arange(psi.size, dtype=np.int64)
    j = np.zeros(psi.size, dtype=np.int64)
    for b, q in enumerate(g_of_reg):
        j |= ((idx >> q) & 1) << b
    n = 1 << len(g_of_reg)
    d = coef[off:off + 2 * n:2] + 1j * coef[off + 1:off + 2 * n:2]
    want = {1: 1.0, 2: -1.0, 3: 1j, 4: -1j}
    for e in range(n):
        c = (codes >> (3 * e)) & 7
        if c:
            assert d[e] == want[c], (e, c, d[e])
    psi *= d[j]


def interpret2(plan, psi, lam):
    """Execute an adjoint sweep plan on (psi, lam); returns the probe values."""
    states = [psi.copy(), lam.copy()]
    vals = np.zeros(len(plan["probe_slots"]))
    coef = plan["coef"]

    def apply_both(kind, t, cm, pm, flags, special, off, tk=()):
        for st in states:
            apply_global(st, kind, t, cm, pm, flags, special, coef, off, tk)

    for pd in plan["passes"]:
        if pd["type"] in (PASS_SMALL, PASS_GLOBALOP):
            for o in plan["ops"][pd["op_begin"]: pd["op_begin"] + pd["op_count"]]:
                if o["kind"] == K_PROBE:
                    vals[o["probe"]] = probe_value(states[0], states[1], int(o["xreg"]), int(o["pthr"]),
                                                   int(o["cthr"]), int(o["special"]), coef[o["coef"]])
                    continue
                tk, pm = kop_targets(o)
                t = (int(o["t0"]), int(o["t1"])) if o["kind"] in (K_SWAP, K_DENSE2) else int(o["t0"])
                apply_both(int(o["kind"]), t, int(o["cthr"]), pm, int(o["flags"]), int(o["special"]),
                           int(o["coef"]), tk)
            continue
        T = int(pd["T"])
        tq = [int(x) for x in pd["tq"][:T]]
        for sd in plan["steps"][pd["step_begin"]: pd["step_begin"] + pd["step_count"]]:
            ops = plan["ops"][sd["op_begin"]: sd["op_begin"] + sd["op_count"]]
            if sd["type"] == STEP_SMEM:
                for o in ops:
                    cm = int(o["cthr"])
                    for b in _bits(o["creg"]):
                        cm |= 1 << tq[b]
                    apply_both(int(o["kind"]), (tq[o["t0"]], tq[o["t1"]]), cm, 0, 0, 0, int(o["coef"]))
                continue
            R = plan["R"]
            g_of_reg = [tq[p] for p in [int(x) for x in sd["rpos"][:R]]]
            for o in ops:
                cm, pm = int(o["cthr"]), int(o["pthr"])
                for b in _bits(o["creg"]):
                    cm |= 1 << g_of_reg[b]
                for b in _bits(o["preg"]):
                    pm |= 1 << g_of_reg[b]
                kind = int(o["kind"])
                if kind == K_PROBE:
                    xm = 0
                    for b in _bits(o["xreg"]):
                        xm |= 1 << g_of_reg[b]
                    vals[int(pd["probe_base"]) + int(o["probe"])] = probe_value(
                        states[0], states[1], xm, pm, cm, int(o["special"]), coef[o["coef"]])
                    continue
                if kind == K_SWAP:
                    t = (g_of_reg[o["t0"]], g_of_reg[o["t1"]])
                elif kind == K_DIAG:
                    t = 0
                else:
                    t = g_of_reg[o["t0"]]
                apply_both(kind, t, cm, pm, int(o["flags"]), int(o["special"]), int(o["coef"]))
    return vals


def interpret(plan, psi):
    """Execute a host plan on a numpy complex128 state and check its
    structural invariants; returns the final state."""
    psi = psi.copy()
    coef = plan["coef"]
    for pd in plan["passes"]:
        if pd["type"] in (PASS_SMALL, PASS_GLOBALOP):
            for o in plan["ops"][pd["op_begin"]: pd["op_begin"] + pd["op_count"]]:
                tk, pm = kop_targets(o)
                t = (int(o["t0"]), int(o["t1"])) if o["kind"] in (K_SWAP, K_DENSE2) else int(o["t0"])
                apply_global(psi, int(o["kind"]), t, int(o["cthr"]), pm, int(o["flags"]),
                             int(o["special"]), coef, int(o["coef"]), tk)
            continue
        T, L = int(pd["T"]), int(pd["L"])
        tq = [int(x) for x in pd["tq"][:T]]
        assert tq[:L] == list(range(L)) and tq == sorted(tq) and len(set(tq)) == T
        for sd in plan["steps"][pd["step_begin"]: pd["step_begin"] + pd["step_count"]]:
            ops = plan["ops"][sd["op_begin"]: sd["op_begin"] + sd["op_count"]]
            if sd["type"] == STEP_SMEM:
                for o in ops:
                    cm = int(o["cthr"])
                    for b in _bits(o["creg"]):
                        cm |= 1 << tq[b]
                    t = (tq[o["t0"]], tq[o["t1"]])
                    apply_global(psi, int(o["kind"]), t, cm, 0, 0, 0, coef, int(o["coef"]))
                continue
            R = plan["R"]
            rpos = [int(x) for x in sd["rpos"][:R]]
            tpos = [int(x) for x in sd["tpos"][: T - R]]
            assert sorted(rpos + tpos) == list(range(T)), (rpos, tpos)
            assert [int(x) for x in sd["tglob"][: T - R]] == [tq[p] for p in tpos]
            eb = plan["elem_bytes"]
            assert [int(x) for x in sd["tsw"][: T - R]] == [tile_off(1 << p, eb) for p in tpos]
            assert [int(x) for x in sd["rsw"][:R]] == [tile_off(1 << p, eb) for p in rpos]
            g_of_reg = [tq[p] for p in rpos]
            for o in ops:
                if int(o["kind"]) == K_DIAGR:
                    apply_diagr(psi, g_of_reg, coef, int(o["coef"]), diagr_codes(o))
                    continue
                cm = int(o["cthr"])
                pm = int(o["pthr"])
                assert bool(int(o["flags"]) & 16) == (cm != 0) and bool(int(o["flags"]) & 32) == (pm != 0)
                assert all(q not in g_of_reg for q in _bits(o["cthr"])), "register qubit in thread control mask"
                for b in _bits(o["creg"]):
                    cm |= 1 << g_of_reg[b]
                for b in _bits(o["preg"]):
                    pm |= 1 << g_of_reg[b]
                kind = int(o["kind"])
                if kind in (K_SWAP,):
                    t = (g_of_reg[o["t0"]], g_of_reg[o["t1"]])
                elif kind == K_DIAG:
                    t = 0
                else:
                    assert o["t0"] < R
                    t = g_of_reg[o["t0"]]
                apply_global(psi, kind, t, cm, pm, int(o["flags"]), int(o["special"]), coef, int(o["coef"]))
    return psi


_INV = {"s": "sdg", "sdg": "s", "t": "tdg", "tdg": "t"}


def dagger(op: ir.Op) -> ir.Op:
    """Inverse of one gate op (for U^dagger U = I property checks)."""
    if op.matrix is not None:
        return ir.Op(op.name, op.kind, op.qubits, op.ncontrols, op.params, matrix=np.asarray(op.matrix).conj().T)
    if op.name in ("rx", "ry", "rz", "p", "cp", "rzz"):
        return ir.Op(op.name, op.kind, op.qubits, op.ncontrols, tuple(-x for x in op.params))
    name = _INV.get(op.name, op.name)
    return ir.Op(name, ir.NAMED_KIND[name], op.qubits, op.ncontrols, op.params)


def inverse(ops):
    return [dagger(o) for o in reversed(ops)]


def random_state(n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return (psi / np.linalg.norm(psi)).astype(np.complex128)


def noise_uniforms(ops, shots, seed, extra_seed=123):
    """The reference's draws per noisy shot (numpy's legacy global generator,
    seeded): one per unitary channel, then one per Kraus channel; then one
    draw for the final sample from a separate generator."""
    nch = sum(1 for o in ops if o.kind in (44, 45))
    np.random.seed(seed)
    extra = np.random.default_rng(extra_seed)
    out = np.zeros((shots, nch + 1))
    for s in range(shots):
        for k in range(nch):
            out[s, k] = np.random.random_sample()
        out[s, nch] = extra.random()
    return out


def noise_terms(pairs):
    """[("X1 Z2", coeff)] -> [(coeff, "XZ", [1, 2])]."""
    terms = []
    for pstr, c in pairs:
        parts = pstr.split()
        terms.append((c, "".join(t[0] for t in parts), [int(t[1:]) for t in parts]))
    return terms
