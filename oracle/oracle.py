"""CPU oracle for the statevector hot path (TEST INFRASTRUCTURE ONLY).

Python driver over ``qsv_oracle.c``: a plain-C restatement of pyquafu's qfvm
complex128 CPU path.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module; the GPU engine in
``pyquafu_gb300`` never does.

Each function cites the reference lines it follows:
  * ``simulate``            src/qfvm/simulator.hpp:115-125 (+ apply_op :30-113)
  * ``expect_statevec``     src/qfvm/qfvm.cpp:246-261, statevector.hpp:1250-1305
  * ``sample_indices``      statevector.hpp:1380-1412 (host-supplied uniforms)
  * ``measure_counts``      statevector.hpp:1398-1409 (bitstring per cbit)
  * ``grad_adjoint``        quafu/algorithms/gradients/gradiant.py:144-173
  * ``grad_adjoint_timing`` the same, timed on a bounded reverse sweep (CPU baseline)
  * ``grad_param_shift``    quafu/algorithms/gradients/gradiant.py:38-73
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "libqsv_oracle.so")

# Named-gate codes (same numbering as QFVM_OP_* in include/qfvm_gb300.h).
NAMED = {
    "x": 1, "y": 2, "z": 3, "h": 4, "s": 5, "sdg": 6, "t": 7, "tdg": 8, "p": 9,
    "rx": 10, "ry": 11, "rz": 12, "cx": 13, "cnot": 13, "cz": 14, "cp": 15,
    "ccx": 16, "rzz": 17,
}


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (portable flags, OpenMP, no FMA contraction)."""
    src = os.path.join(_HERE, "qsv_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11",
               src, "-o", _SO, "-lm"]
        subprocess.check_call(cmd)
    return _SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        u64 = ctypes.c_uint64
        L.qor_apply_named.argtypes = [dp, u64, ctypes.c_int, ip, dp]
        L.qor_apply_named.restype = ctypes.c_int
        L.qor_apply_matrix.argtypes = [dp, u64, ip, ctypes.c_int, ctypes.c_int, dp]
        L.qor_apply_matrix.restype = ctypes.c_int
        L.qor_expect_pauli.argtypes = [dp, u64, u64, u64, ctypes.c_int]
        L.qor_expect_pauli.restype = ctypes.c_double
        L.qor_sample_indices.argtypes = [dp, u64, dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
        L.qor_sequential_cdf.argtypes = [dp, u64, dp]
        L.qor_sample_indices_sorted.argtypes = [dp, u64, dp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int64,
                                                ctypes.POINTER(ctypes.c_uint64)]
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def zero_state(n: int) -> np.ndarray:
    """|0...0>: StateVector(num) constructor, statevector.hpp:148-152."""
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    return psi


def apply_op(psi: np.ndarray, op) -> np.ndarray:
    """apply_op (simulator.hpp:30-113) for one gate of the packed IR, in place.

    ``op`` is a ``pyquafu_gb300.ir.Op``-like object with ``name``, ``qubits``
    (controls first), ``ncontrols``, ``params`` and ``matrix``.
    """
    assert psi.dtype == np.complex128 and psi.flags.c_contiguous
    L = lib()
    q = np.ascontiguousarray(op.qubits, dtype=np.int32)
    qp = q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    if op.name in NAMED and op.matrix is None:
        par = np.ascontiguousarray(list(op.params) + [0.0], dtype=np.float64)
        rc = L.qor_apply_named(_dptr(psi.view(np.float64)), psi.size, NAMED[op.name], qp, _dptr(par))
    else:
        m = np.ascontiguousarray(op.matrix, dtype=np.complex128)
        rc = L.qor_apply_matrix(_dptr(psi.view(np.float64)), psi.size, qp, len(q), op.ncontrols,
                                _dptr(m.view(np.float64)))
    if rc != 0:
        raise RuntimeError(f"oracle: cannot apply {op.name}")
    return psi


def simulate(n: int, ops, psi: np.ndarray | None = None) -> np.ndarray:
    """simulate(): simulator.hpp:115-125 over the gate ops (measures skipped)."""
    if psi is None or psi.size == 0:
        psi = zero_state(n)
    else:
        psi = np.ascontiguousarray(psi, dtype=np.complex128).copy()
    for op in ops:
        apply_op(psi, op)
    return psi


# ------------------------------------------------------------------
# Circuits with mid-circuit measurement, reset and classically controlled
# blocks: the per-shot branch of simulate_circuit (qfvm.cpp:104-133).  The
# reference draws each outcome with std::discrete_distribution over an
# rng seeded from std::random_device (statevector.hpp:1307-1341); here every
# measure/reset consumes one given uniform u and picks the first outcome m
# with u * total < cum[m], probabilities summed in FP64 in index order.
# ------------------------------------------------------------------


def _outcome_probs(psi, qbits):
    """sample_measure_probs (statevector.hpp:1307-1341): probability of every
    joint outcome m of qbits (bit j of m <-> qbits[j])."""
    idx = np.arange(psi.size, dtype=np.int64)
    m = np.zeros(psi.size, dtype=np.int64)
    for j, q in enumerate(qbits):
        m |= ((idx >> q) & 1) << j
    p = (psi.real * psi.real + psi.imag * psi.imag)
    probs = np.zeros(1 << len(qbits))
    for k in range(probs.size):  # index order inside every outcome
        sel = p[m == k]
        acc = 0.0
        for v in sel:
            acc += float(v)
        probs[k] = acc
    return probs, m


def choose_outcome(probs, u):
    """First outcome m with u * total < cum[m] (FP64, outcome order); the
    last outcome of nonzero probability when rounding leaves none."""
    total = 0.0
    for v in probs:
        total += float(v)
    r = float(u) * total
    cum = 0.0
    last = 0
    for k, v in enumerate(probs):
        cum += float(v)
        if v > 0:
            last = k
        if r < cum:
            return k
    return last


def _collapse(psi, qbits, m_of, outcome, prob, final):
    """update (statevector.hpp:1192-1225): keep outcome, scale 1/sqrt(prob),
    then move it to `final` (reset) by exchanging the two outcome blocks."""
    scale = 1.0 / np.sqrt(prob)
    keep = m_of == outcome
    out = np.where(keep, psi * scale, 0)
    if final != outcome:
        moved = np.zeros_like(out)
        delta = 0
        for j, q in enumerate(qbits):
            if ((outcome ^ final) >> j) & 1:
                delta |= 1 << q
        idx = np.arange(psi.size, dtype=np.int64)
        moved[idx[keep] ^ delta] = out[keep]
        out = moved
    psi[:] = out


def run_shot(n, ops, ncbits, uniforms, psi_in=None):
    """One shot of the per-shot branch: returns (creg list, final state)."""
    psi = zero_state(n) if psi_in is None or np.size(psi_in) == 0 else np.array(psi_in, dtype=np.complex128)
    creg = [0] * max(ncbits, 1)
    draw = 0

    def run(seq):
        nonlocal draw
        for op in seq:
            if op.kind == 40 or op.kind == 41:  # measure / reset
                probs, m_of = _outcome_probs(psi, op.qbits)
                k = choose_outcome(probs, uniforms[draw])
                draw += 1
                _collapse(psi, op.qbits, m_of, k, probs[k], 0 if op.kind == 41 else k)
                if op.kind == 40:
                    for j, c in enumerate(op.cbits):
                        creg[c] = (k >> j) & 1
            elif op.kind == 42:  # cif: check_cif (statevector.hpp:186-193)
                out = 0
                for c in op.cbits:
                    out = out * 2 + creg[c]
                if out == op.condition:
                    run(op.body)
            elif op.kind == 43:
                continue
            else:
                apply_op(psi, op)

    run(ops)
    return creg, psi


def simulate_shots(n, ops, ncbits, uniforms, psi_in=None):
    """Per-shot loop of qfvm.cpp:104-133: outcome of every shot (measured
    cbits in ascending order, the first one most significant) and the final
    state of the last shot.  uniforms[s] holds shot s's draws in order."""
    measured = sorted({c for op in _walk(ops) if op.kind == 40 for c in op.cbits})
    outcomes = []
    psi = None
    for s in range(len(uniforms)):
        creg, psi = run_shot(n, ops, ncbits, uniforms[s], psi_in)
        v = 0
        for c in measured:
            v = v * 2 + creg[c]
        outcomes.append(v)
    return outcomes, psi


# ------------------------------------------------------------------
# Noisy trajectories: NoiseSVSimulator (quafu/simulators/simulator.py:148-225).
# Per shot the reference draws one number per unitary channel while building
# the sampled circuit (gen_circuit, :196-218, np.random.choice), then one per
# Kraus channel while running it (_apply_op, :61-76, np.random.rand), then
# samples one index (sampling_statevec); here those draws are given uniforms
# in the same order.
# ------------------------------------------------------------------


def _apply_1q(psi, q, m):
    from types import SimpleNamespace

    apply_op(psi, SimpleNamespace(name="kraus_op", qubits=(q,), ncontrols=0, params=(), matrix=np.asarray(m)))


def run_noisy_shot(n, ops, uniforms, psi_in=None):
    """One shot: (sampled basis index, final state)."""
    psi = zero_state(n) if psi_in is None or np.size(psi_in) == 0 else np.array(psi_in, dtype=np.complex128)
    nu = sum(1 for o in ops if o.kind == 44)
    iu, ik = 0, nu
    for op in ops:
        if op.kind == 44:  # UnitaryChannel.gen_gate: np.random.choice(gatelist, p=probs)
            cdf = np.cumsum(np.asarray(op.params, dtype=np.float64))
            cdf /= cdf[-1]
            i = int(np.searchsorted(cdf, uniforms[iu], side="right"))
            iu += 1
            _apply_1q(psi, op.qubits[0], op.matrix[min(i, len(cdf) - 1)])
        elif op.kind == 45:  # KrausChannel in _apply_op: s += ||K psi|| / ||psi||
            r = uniforms[ik]
            ik += 1
            norm0 = np.linalg.norm(psi)
            s = 0.0
            for k in op.matrix:
                t = psi.copy()
                _apply_1q(t, op.qubits[0], k)
                norm1 = np.linalg.norm(t)
                s += norm1 / norm0
                if r < s:
                    psi[:] = t / norm1
                    break
        elif op.kind == 43:
            continue
        else:
            apply_op(psi, op)
    idx = int(sample_indices(psi, np.array([uniforms[len(uniforms) - 1]]))[0])
    return idx, psi


def simulate_noise(n, ops, uniforms, psi_in=None, terms=None):
    """NoiseSVSimulator.run: per shot the sampled index and, with terms
    [(coeff, paulistr, pos)], coeff * <P> of the shot's final state."""
    samples, expv = [], []
    for u in uniforms:
        idx, psi = run_noisy_shot(n, ops, u, psi_in)
        samples.append(idx)
        if terms:
            expv.append([c * expect_pauli(psi, p, pos) for c, p, pos in terms])
    return samples, (np.array(expv) if terms else None)


def _walk(ops):
    for op in ops:
        yield op
        if op.kind == 42:
            yield from _walk(op.body)


def pauli_masks(paulistr: str, pos) -> tuple[int, int, int]:
    """Flip/Z masks and Y count as in statevector.hpp:1252-1279."""
    xm = zm = 0
    ny = 0
    for ch, q in zip(paulistr, pos):
        if ch == "X":
            xm |= 1 << q
        elif ch == "Y":
            xm |= 1 << q
            zm |= 1 << q
            ny += 1
        elif ch == "Z":
            zm |= 1 << q
    return xm, zm, ny


def expect_pauli(psi: np.ndarray, paulistr: str, pos) -> float:
    xm, zm, ny = pauli_masks(paulistr, pos)
    return lib().qor_expect_pauli(_dptr(psi.view(np.float64)), psi.size, xm, zm, ny)


def expect_statevec(psi: np.ndarray, paulis) -> list[float]:
    """expect_statevec: qfvm.cpp:246-261 (unweighted per-term values)."""
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    return [expect_pauli(psi, p.paulistr, p.pos) for p in paulis]


def sample_indices(psi: np.ndarray, uniforms: np.ndarray) -> np.ndarray:
    """Sequential FP64 CDF scan of measure_samples (statevector.hpp:1387-1397)."""
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    out = np.zeros(u.size, dtype=np.uint64)
    lib().qor_sample_indices(_dptr(psi.view(np.float64)), psi.size, _dptr(u), u.size,
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out


def sample_indices_sorted(psi: np.ndarray, uniforms: np.ndarray) -> np.ndarray:
    """The indices of sample_indices from one walk of the FP64 running sum
    (shots visited by ascending uniform): O(size + shots) instead of
    O(size * shots), the same sums and comparisons."""
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    order = np.ascontiguousarray(np.argsort(u, kind="stable"), dtype=np.int64)
    out = np.zeros(u.size, dtype=np.uint64)
    lib().qor_sample_indices_sorted(_dptr(psi.view(np.float64)), psi.size, _dptr(u),
                                    order.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), u.size,
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out


def sequential_cdf(psi: np.ndarray) -> np.ndarray:
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    cdf = np.empty(psi.size, dtype=np.float64)
    lib().qor_sequential_cdf(_dptr(psi.view(np.float64)), psi.size, _dptr(cdf))
    return cdf


def bitstrings(indices, measures) -> list[str]:
    """Bitstring per shot: char at cbit index = bit (sample >> qbit) & 1
    (statevector.hpp:1398-1401). ``measures`` is a list of (qbit, cbit)."""
    nb = len(measures)
    out = []
    for s in indices:
        s = int(s)
        b = ["0"] * nb
        for q, c in measures:
            b[c] = "1" if (s >> q) & 1 else "0"
        out.append("".join(b))
    return out


def measure_counts(psi, measures, uniforms) -> dict:
    """measure_samples (statevector.hpp:1380-1412) driven by given uniforms."""
    counts: dict = {}
    for b in bitstrings(sample_indices(psi, uniforms), measures):
        counts[b] = counts.get(b, 0) + 1
    return counts


# ----------------------------- gradients -----------------------------

_PAULI = {
    "X": np.array([[0, 1], [1, 0]], dtype=complex),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=complex),
    "Z": np.array([[1, 0], [0, -1]], dtype=complex),
}


def _rot_matrix(name, theta):
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    if name == "rx":
        return np.array([[c, -1j * s], [-1j * s, c]])
    if name == "ry":
        return np.array([[c, -s], [s, c]], dtype=complex)
    return np.array([[np.exp(-0.5j * theta), 0], [0, np.exp(0.5j * theta)]])


def apply_hamiltonian(psi, terms) -> np.ndarray:
    """_apply_hamil (quafu/simulators/simulator.py:156-166): sum_k c_k P_k psi.
    ``terms`` is a list of (coeff, paulistr, pos)."""
    from types import SimpleNamespace

    out = np.zeros_like(psi)
    for coeff, pstr, pos in terms:
        p1 = psi.copy()
        for ch, q in zip(pstr, pos):
            apply_op(p1, SimpleNamespace(name=ch.lower(), qubits=(q,), ncontrols=0, params=(), matrix=None))
        out += p1 * coeff
    return out


def _dagger(op):
    """op.dagger(): rotations negate the angle, fixed gates use the inverse."""
    from types import SimpleNamespace

    inv = {"s": "sdg", "sdg": "s", "t": "tdg", "tdg": "t"}
    if op.matrix is not None:
        m = np.asarray(op.matrix).conj().T
        return SimpleNamespace(name=op.name, qubits=op.qubits, ncontrols=op.ncontrols, params=(), matrix=m)
    if op.name in ("rx", "ry", "rz", "p", "cp", "rzz"):
        return SimpleNamespace(name=op.name, qubits=op.qubits, ncontrols=op.ncontrols,
                               params=tuple(-x for x in op.params), matrix=None)
    return SimpleNamespace(name=inv.get(op.name, op.name), qubits=op.qubits, ncontrols=op.ncontrols,
                           params=op.params, matrix=None)


def _grad_gate(op):
    """grad_gate (gradiant.py:96-141): -i/2 * P * G as a matrix gate; controlled
    rotations get a projector on the controls."""
    from types import SimpleNamespace

    base = op.name[-2:]  # rx / ry / rz (also crx, cry, crz, mcrx ...)
    P = _PAULI[base[1].upper()]
    G = _rot_matrix(base, op.params[0])
    d = -0.5j * P @ G
    return SimpleNamespace(name="d" + base, qubits=op.qubits, ncontrols=op.ncontrols, params=(), matrix=d)


def grad_adjoint(n, ops, param_index, terms, psi_in=None):
    """Adjoint gradient (gradiant.py:144-173): reverse sweep un-applying gates to
    phi and lam; grad_i = Re 2 <lam| dG_i |phi>.  ``param_index[i]`` is the
    trainable-parameter slot of gate i, or -1.  Returns d<H>/d(slot)."""
    phi = simulate(n, ops, psi_in)
    lam = apply_hamiltonian(phi, terms)
    nslot = max([k for k in param_index if k >= 0], default=-1) + 1
    grads = np.zeros(nslot)
    for i in range(len(ops) - 1, -1, -1):
        op = ops[i]
        apply_op(phi, _dagger(op))
        if param_index[i] >= 0:
            mu = phi.copy()
            g = _grad_gate(op)
            if op.ncontrols:
                # projector on the controls: controlled derivative acts only
                # where every control is 1 (gradiant.py:99-131)
                mask = 0
                for c in op.qubits[: op.ncontrols]:
                    mask |= 1 << c
                idx = np.arange(mu.size)
                tmp = mu.copy()
                apply_op(tmp, type(g)(name=g.name, qubits=op.qubits[op.ncontrols:], ncontrols=0,
                                      params=(), matrix=g.matrix))
                sel = (idx & mask) == mask
                mu = np.where(sel, tmp, 0)
            else:
                apply_op(mu, g)
            grads[param_index[i]] += np.real(2.0 * np.vdot(lam, mu))
        apply_op(lam, _dagger(op))
    return grads


def grad_adjoint_timing(n, ops, param_index, terms, seconds):
    """grad_adjoint above, timed for the CPU baseline: the forward
    simulation and lam = H psi in full, then the reverse sweep until
    `seconds` have elapsed.  Returns (forward s, lam s, reverse gates done,
    reverse s)."""
    import time

    t0 = time.perf_counter()
    phi = simulate(n, ops)
    t1 = time.perf_counter()
    lam = apply_hamiltonian(phi, terms)
    t2 = time.perf_counter()
    done = 0
    for i in range(len(ops) - 1, -1, -1):
        op = ops[i]
        apply_op(phi, _dagger(op))
        if param_index[i] >= 0 and not op.ncontrols:
            mu = phi.copy()
            apply_op(mu, _grad_gate(op))
            np.real(2.0 * np.vdot(lam, mu))
        apply_op(lam, _dagger(op))
        done += 1
        if time.perf_counter() - t2 > seconds:
            break
    return t1 - t0, t2 - t1, done, time.perf_counter() - t2


def energy(n, ops, terms, psi_in=None) -> float:
    psi = simulate(n, ops, psi_in)
    e = 0.0
    for coeff, pstr, pos in terms:
        e += coeff * expect_pauli(psi, pstr, pos)
    return e


def grad_param_shift(n, ops, param_index, terms, psi_in=None):
    """Parameter shift (gradiant.py:38-73): (f(t+pi/2) - f(t-pi/2)) / 2 for each
    parameterised rx/ry/rz occurrence, summed into its slot."""
    from types import SimpleNamespace

    nslot = max([k for k in param_index if k >= 0], default=-1) + 1
    grads = np.zeros(nslot)
    for i, op in enumerate(ops):
        if param_index[i] < 0:
            continue
        res = []
        for sh in (np.pi / 2, -np.pi / 2):
            shifted = list(ops)
            shifted[i] = SimpleNamespace(name=op.name, qubits=op.qubits, ncontrols=op.ncontrols,
                                         params=(op.params[0] + sh,) + tuple(op.params[1:]), matrix=None)
            res.append(energy(n, shifted, terms, psi_in))
        grads[param_index[i]] += (res[0] - res[1]) / 2.0
    return grads


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(_SO)
