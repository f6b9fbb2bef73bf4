"""Drop-in replacement for pyquafu's ``qfvm`` pybind module on the GB300 engine.

Same function names, argument meaning, return values and in-place semantics as
src/qfvm/qfvm.cpp:263-288; the gates run on the GPU through the C ABI of
include/qfvm_gb300.h.  Install it where pyquafu imports its native module::

    import sys, pyquafu_gb300.qfvm as q
    sys.modules["quafu.simulators.qfvm"] = q      # before importing quafu

The reference draws sampling uniforms from ``std::random_device``
(util.h:35-45); this module draws them from a NumPy generator that
``set_seed`` makes reproducible.  The uniforms used by the last call are kept
in ``last_uniforms`` so a run can be replayed against the CPU scan.
"""

from __future__ import annotations

import numpy as np

from . import _native as nat
from . import ir

__all__ = [
    "simulate_circuit", "applyop_statevec", "sampling_statevec", "expect_statevec",
    "simulate_circuit_gpu", "simulate_circuit_custate", "simulate_circuit_clifford",
    "set_seed", "QfvmError",
]

QfvmError = nat.QfvmError
_rng = np.random.default_rng()
last_uniforms: np.ndarray = np.zeros(0)


def set_seed(seed) -> None:
    """Make the sampling uniforms reproducible (no counterpart in the reference)."""
    global _rng
    _rng = np.random.default_rng(seed)


def set_arithmetic(kind: str) -> None:
    """Arithmetic of this module's complex128 work (no counterpart in the
    reference): "ds" (float pairs on the FP32 pipes, the default;
    per-amplitude error below 1e-12 against FP64) or "fp64" (IEEE FP64).
    The state stays complex128 either way."""
    codes = {"ds": nat.QFVM_C128_DS, "fp64": nat.QFVM_C128}
    if kind not in codes:
        raise ValueError(f"arithmetic must be 'ds' or 'fp64', not {kind!r}")
    nat.check(nat.load().qfvm_set_c128_arithmetic(codes[kind]), "set_arithmetic")


def get_arithmetic() -> str:
    return "ds" if nat.load().qfvm_get_c128_arithmetic() == nat.QFVM_C128_DS else "fp64"


def _uniforms(shots: int) -> np.ndarray:
    global last_uniforms
    last_uniforms = _rng.random(int(shots))
    return last_uniforms


def _as_state(inputstate) -> np.ndarray:
    """py::array_t<complex<double>> conversion: reuse the caller's array when it
    already is contiguous complex128 (so updates are in place), else copy."""
    if inputstate is None:
        return np.zeros(0, dtype=np.complex128)
    arr = np.asarray(inputstate)
    if arr.dtype == np.complex128 and arr.flags.c_contiguous and arr.ndim == 1:
        return arr
    return np.ascontiguousarray(arr, dtype=np.complex128).reshape(-1)


def _qubits_of(size: int) -> int:
    n = int(size).bit_length() - 1
    if size < 2 or (1 << n) != size:
        raise QfvmError(f"state length {size} is not a power of two >= 2")
    return n


def _bitstrings(indices, measures) -> list[str]:
    """statevector.hpp:1388-1401: char at cbit index = bit (sample >> qbit) & 1."""
    nb = len(measures)
    for _, c in measures:
        if c >= nb:
            # std::string::replace past the end throws in the reference
            raise QfvmError(f"classical bit {c} outside a {nb}-bit measurement string")
    idx = np.asarray(indices, dtype=np.uint64)
    chars = np.full((idx.size, nb), ord("0"), dtype=np.uint8)
    for q, c in measures:
        chars[:, c] = ord("0") + ((idx >> np.uint64(q)) & np.uint64(1)).astype(np.uint8)
    return [row.tobytes().decode("ascii") for row in chars]


def _count(strings) -> dict:
    counts: dict = {}
    for s in strings:
        counts[s] = counts.get(s, 0) + 1
    return counts


def _gate_ops(ops):
    return [op for op in ops if op.is_gate and op.kind != ir.OP_NOP]


def _has_classical(ops) -> bool:
    return any(op.kind in (ir.OP_RESET, ir.OP_CIF) for op in ops)


def _shots(n: int, ncbits: int, ops, psi: np.ndarray, shots: int):
    """qfvm_simulate_shots: every shot's outcome and the last shot's state."""
    for op in ops:
        if op.is_gate:
            ir.validate([op], n)
        elif op.kind == ir.OP_CIF:
            ir.validate([b for b in op.body if b.is_gate and b.kind != ir.OP_NOP], n)
    arr, pool = ir.pack_program(ops)
    nd = ir.program_draws(ops)
    uni = _uniforms(shots * nd) if nd else np.zeros(1)
    out = np.zeros(shots, dtype=np.uint64)
    final = np.empty(1 << n, dtype=np.complex128)
    psi_p = nat.dptr(psi.view(np.float64)) if psi.size else None
    rc = nat.load().qfvm_simulate_shots(n, int(ncbits), nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                                        pool.size, psi_p, int(shots), nat.dptr(uni), nd, nat.u64ptr(out),
                                        nat.dptr(final.view(np.float64)))
    nat.check(rc, "simulate_circuit (per-shot trajectories)")
    return out, final


def _run(n: int, ops, state: np.ndarray, given: bool, shots: int) -> np.ndarray:
    lib = nat.load()
    arr, pool = ir.pack(ops)
    uni = _uniforms(shots) if shots > 0 else np.zeros(1)
    idx = np.zeros(max(shots, 1), dtype=np.uint64)
    rc = lib.qfvm_simulate_circuit(n, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)), pool.size,
                                   nat.dptr(state.view(np.float64)), 1 if given else 0, nat.dptr(uni),
                                   int(shots), nat.u64ptr(idx))
    nat.check(rc, "simulate_circuit")
    return idx[:shots]


def simulate_circuit(circuit, inputstate=None, shots=None):
    """qfvm.cpp:68-134.  Returns (counts {int: int}, statevector)."""
    if shots is None:
        raise TypeError("simulate_circuit() missing required argument 'shots'")
    shots = int(shots)
    circ = ir.read_circuit(circuit)
    psi = _as_state(inputstate)
    given = psi.size != 0
    n = _qubits_of(psi.size) if given else circ.num_qubits
    if n < 1:
        raise QfvmError("a circuit needs at least one qubit")
    if not circ.final_measure:
        # per-shot branch (qfvm.cpp:104-133): one trajectory per shot; the
        # returned state is the last shot's
        if shots < 1:
            raise QfvmError("circuits with operations after a measurement need shots >= 1", 1)
        out, final = _shots(n, circ.cbits_num, circ.ops, psi, shots)
        counts: dict = {}
        for v in out.tolist():
            counts[int(v)] = counts.get(int(v), 0) + 1
        return counts, final
    if _has_classical(circ.ops):
        # measures only at the end but resets / cifs before them: one
        # trajectory with the measures skipped (simulator.hpp:115-125), then
        # the counts are sampled from its state as for any final measurement
        prog = [op for op in circ.ops if op.kind != ir.OP_MEASURE]
        _, final = _shots(n, circ.cbits_num, prog, psi, 1)
        state = psi if given else final
        if given:
            state[:] = final
        measures = circ.measure_vec
        outcount: dict = {}
        if measures and shots > 0:
            idx = np.zeros(shots, dtype=np.uint64)
            uni = _uniforms(shots)
            nat.check(nat.load().qfvm_sampling_statevec(nat.dptr(state.view(np.float64)), state.size,
                                                        nat.dptr(uni), shots, nat.u64ptr(idx)), "sampling")
            for s_, c in _count(_bitstrings(idx, measures)).items():
                outcount[int(s_, 2)] = c
        return outcount, state
    ops = _gate_ops(circ.ops)
    ir.validate(ops, n)
    state = psi if given else np.empty(1 << n, dtype=np.complex128)
    measures = circ.measure_vec
    nshots = shots if measures else 0
    idx = _run(n, ops, state, given, nshots)
    outcount: dict = {}
    if measures:
        for s, c in _count(_bitstrings(idx, measures)).items():
            outcount[int(s, 2)] = c  # qfvm.cpp:95 stoi(bitstring, 2)
    return outcount, state


def simulate_circuit_gpu(circuit, inputstate=None):
    """qfvm.cpp:207-223: simulate and return the statevector only."""
    circ = ir.read_circuit(circuit)
    psi = _as_state(inputstate)
    given = psi.size != 0
    n = _qubits_of(psi.size) if given else circ.num_qubits
    ops = _gate_ops(circ.ops)
    ir.validate(ops, n)
    state = psi if given else np.empty(1 << n, dtype=np.complex128)
    _run(n, ops, state, given, 0)
    return state


simulate_circuit_custate = simulate_circuit_gpu


def applyop_statevec(operation, inputstate):
    """qfvm.cpp:36-50: apply one gate to the state in place and return it."""
    psi = _as_state(inputstate)
    op = ir.read_op(operation)
    if psi.size == 0 or op is None:
        return psi
    if not op.is_gate:
        raise QfvmError(f"'{op.name}' is not supported by applyop_statevec on the GB300 engine", 4)
    if op.kind == ir.OP_NOP:
        return psi
    n = _qubits_of(psi.size)
    ir.validate([op], n)
    arr, pool = ir.pack([op])
    rc = nat.load().qfvm_applyop_statevec(nat.vptr(arr), nat.dptr(pool.view(np.float64)), pool.size,
                                         nat.dptr(psi.view(np.float64)), psi.size)
    nat.check(rc, "applyop_statevec")
    return psi


def sampling_statevec(measures, inputstate, shots):
    """qfvm.cpp:52-66: {bitstring: count} with bit (sample >> qbit) at cbit."""
    psi = _as_state(inputstate)
    meas = [(int(q), int(c)) for q, c in dict(measures).items()]
    shots = int(shots)
    if shots <= 0:
        return {}
    _qubits_of(psi.size)
    uni = _uniforms(shots)
    idx = np.zeros(shots, dtype=np.uint64)
    rc = nat.load().qfvm_sampling_statevec(nat.dptr(psi.view(np.float64)), psi.size, nat.dptr(uni), shots,
                                          nat.u64ptr(idx))
    nat.check(rc, "sampling_statevec")
    return _count(_bitstrings(idx, meas))


def expect_statevec(inputstate, paulis):
    """qfvm.cpp:246-261: unweighted <P> per Pauli term (objects with .pos and .paulistr)."""
    from .engine import pack_terms

    psi = _as_state(inputstate)
    terms = [(p.paulistr, list(p.pos)) for p in paulis]
    if not terms:
        return []
    _qubits_of(psi.size)
    x, z, y = pack_terms(terms)
    out = np.zeros(len(terms), dtype=np.float64)
    rc = nat.load().qfvm_expect_statevec(nat.dptr(psi.view(np.float64)), psi.size, nat.u64ptr(x), nat.u64ptr(z),
                                        nat.i32ptr(y), len(terms), nat.dptr(out))
    nat.check(rc, "expect_statevec")
    return [float(v) for v in out]


def simulate_circuit_clifford(circuit, shots):
    """The stabilizer simulator (src/qfvm_clifford) is outside this engine."""
    raise QfvmError("simulate_circuit_clifford is not provided by the GB300 statevector engine", 4)
