"""Circuit reader: pyquafu circuit objects -> packed gate list for the engine.

Reads the same Python object protocol as the reference's C++ IR builder
(src/qfvm/circuit.hpp:98-135 ``Circuit::Circuit(py::object)`` and
src/qfvm/instructions.hpp:229-299 ``from_pyops``):

* circuit: ``.instructions``, ``.num``, ``.cbits_num``
* gate: ``.name`` (lower-cased), ``.pos`` (controls first), ``._paras``,
  ``.ctrls`` (its length is the control count); for names outside the named
  table (OPMAP, src/qfvm/qasm.hpp:43-46) the target matrix comes from
  ``._get_targ_matrix(reverse_order=True)`` when the gate has ``_targ_matrix``,
  else from ``.matrix``
* oracle / wrapped circuits (objects with ``.circuit``) are flattened
* ``barrier``, ``delay`` and ``id`` are dropped; ``measure`` records
  (qbit, cbit) pairs; any non-measure instruction after a measure clears
  ``final_measure`` (circuit.hpp:447-459)

The packed form (``pack``) is the ``qfvm_op`` array declared in
include/qfvm_gb300.h plus a pool of complex128 matrix entries.
"""

from __future__ import annotations

import numpy as np

# OPMAP (src/qfvm/qasm.hpp:43-46) -> QFVM_OP_* codes of include/qfvm_gb300.h
OP_X, OP_Y, OP_Z, OP_H, OP_S, OP_SDG, OP_T, OP_TDG, OP_P = 1, 2, 3, 4, 5, 6, 7, 8, 9
OP_RX, OP_RY, OP_RZ, OP_CX, OP_CZ, OP_CP, OP_CCX, OP_RZZ = 10, 11, 12, 13, 14, 15, 16, 17
OP_MATRIX = 32
OP_MEASURE, OP_RESET, OP_CIF, OP_NOP = 40, 41, 42, 43
OP_UCHANNEL, OP_KRAUS = 44, 45  # noise channels (qfvm_simulate_noise)

NAMED_KIND = {
    "x": OP_X, "y": OP_Y, "z": OP_Z, "h": OP_H, "s": OP_S, "sdg": OP_SDG, "t": OP_T,
    "tdg": OP_TDG, "p": OP_P, "rx": OP_RX, "ry": OP_RY, "rz": OP_RZ, "cnot": OP_CX,
    "cx": OP_CX, "cz": OP_CZ, "cp": OP_CP, "ccx": OP_CCX, "rzz": OP_RZZ,
}
# names in OPMAP that are not gates (qasm.hpp:43-46)
OPMAP_CLASSIC = {"creg": OP_NOP, "measure": OP_MEASURE, "reset": OP_RESET, "cif": OP_CIF}
OPMAP_NAMES = set(NAMED_KIND) | set(OPMAP_CLASSIC)
SKIPPED = {"barrier", "delay", "id"}

MAX_OP_QUBITS = 16

# generators of parameterised matrix gates (QFVM_GEN_* of include/qfvm_gb300.h)
GEN_NONE, GEN_X, GEN_Y, GEN_Z, GEN_PHASE = 0, 1, 2, 3, 4


def generator_of(name: str, kind: int) -> int:
    """dG/dtheta = -i/2 Q G for the rotation families pyquafu defines
    (element_gates.py: RX/RY/RZ, RXX/RYY/RZZ, CRX/CRY/CRZ, MCRX/MCRY/MCRZ,
    P/CP); named OPMAP gates carry their generator implicitly."""
    if kind != OP_MATRIX:
        return GEN_NONE
    n = name.lower()
    if n.endswith("rx") or n.endswith("rxx"):
        return GEN_X
    if n.endswith("ry") or n.endswith("ryy"):
        return GEN_Y
    if n.endswith("rz") or n.endswith("rzz"):
        return GEN_Z
    if n in ("p", "cp", "mcp", "phase"):
        return GEN_PHASE
    return GEN_NONE

# numpy mirror of ``qfvm_op`` (include/qfvm_gb300.h); 128 bytes, 8-byte aligned
OP_DTYPE = np.dtype(
    [
        ("kind", "<i4"),
        ("ncontrols", "<i4"),
        ("nqubits", "<i4"),
        ("mat_dim", "<i4"),
        ("qubits", "<i4", (MAX_OP_QUBITS,)),
        ("slot", "<i4"),
        ("gen", "<i4"),
        ("params", "<f8", (4,)),
        ("mat_offset", "<i8"),
    ],
    align=True,
)
assert OP_DTYPE.itemsize == 128


class Op:
    """One instruction of the packed list (a gate, or a measure/reset/cif)."""

    __slots__ = ("name", "kind", "qubits", "ncontrols", "params", "matrix", "slot", "gen",
                 "qbits", "cbits", "condition", "body")

    def __init__(self, name, kind, qubits=(), ncontrols=0, params=(), matrix=None, slot=-1,
                 qbits=(), cbits=(), condition=0, body=(), gen=None):
        self.name = name
        self.kind = kind
        self.qubits = tuple(int(q) for q in qubits)
        self.ncontrols = int(ncontrols)
        self.params = tuple(float(p) for p in params)
        self.matrix = matrix
        self.slot = int(slot)
        self.gen = generator_of(name, kind) if gen is None else int(gen)
        self.qbits = tuple(int(q) for q in qbits)
        self.cbits = tuple(int(c) for c in cbits)
        self.condition = int(condition)
        self.body = tuple(body)

    @property
    def is_gate(self) -> bool:
        return self.kind < OP_MEASURE

    def __repr__(self):
        return f"Op({self.name}, q={self.qubits}, c={self.ncontrols}, p={self.params})"


class Circuit:
    """Result of reading a circuit: the reference's ``Circuit`` fields."""

    def __init__(self, num_qubits: int, cbits_num: int):
        self.num_qubits = int(num_qubits)
        self.cbits_num = int(cbits_num)
        self.ops: list[Op] = []
        self.measure_vec: list[tuple[int, int]] = []
        self.final_measure = True

    @property
    def gates(self) -> list[Op]:
        return [o for o in self.ops if o.is_gate]


def _matrix_of(pyop) -> np.ndarray:
    # instructions.hpp:250-255
    if hasattr(pyop, "_targ_matrix"):
        m = pyop._get_targ_matrix(reverse_order=True)
    else:
        m = pyop.matrix
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if m.ndim != 2 or m.shape[0] != m.shape[1]:
        raise ValueError(f"gate {pyop.name}: matrix must be square, got shape {m.shape}")
    return m


def read_op(pyop) -> Op | None:
    """from_pyops (instructions.hpp:229-299).  Returns None for dropped ops."""
    name = str(pyop.name).lower()
    if name in SKIPPED:
        return None
    if name == "measure":
        return Op(name, OP_MEASURE, qbits=list(pyop.qbits), cbits=list(pyop.cbits))
    if name == "reset":
        return Op(name, OP_RESET, qbits=list(pyop.pos))
    if name == "cif":
        body = []
        ins = getattr(pyop, "instructions", None)
        if isinstance(ins, list):
            for sub in ins:
                o = read_op(sub)
                if o is not None:
                    body.append(o)
        return Op(name, OP_CIF, cbits=list(pyop.cbits), condition=int(pyop.condition), body=body)
    pos = list(pyop.pos) if not isinstance(pyop.pos, (int, np.integer)) else [int(pyop.pos)]
    paras = [float(p) for p in pyop._paras]
    ncontrols = len(pyop.ctrls) if hasattr(pyop, "ctrls") else 0
    if name in NAMED_KIND:
        return Op(name, NAMED_KIND[name], pos, ncontrols, paras)
    if name in OPMAP_CLASSIC:  # "creg": named but applies nothing
        return Op(name, OP_NOP, pos, ncontrols, paras)
    return Op(name, OP_MATRIX, pos, ncontrols, paras, matrix=_matrix_of(pyop))


def read_circuit(pycircuit) -> Circuit:
    """Circuit::Circuit(py::object) (circuit.hpp:98-135)."""
    circ = Circuit(int(pycircuit.num), int(pycircuit.cbits_num))
    measured = False
    for pyop in pycircuit.instructions:
        if hasattr(pyop, "circuit"):  # oracle / wrapper: flatten its instructions
            circ.ops.extend(read_circuit(pyop.circuit).ops)
            continue
        op = read_op(pyop)
        if op is None:
            continue
        if op.kind == OP_MEASURE:
            measured = True
            circ.measure_vec.extend(zip(op.qbits, op.cbits))
        elif measured:
            circ.final_measure = False
        circ.ops.append(op)
    return circ


def validate(ops, num_qubits: int) -> None:
    """Host-side checks before anything reaches the device."""
    for op in ops:
        if not op.is_gate:
            continue
        if op.kind == OP_NOP:
            continue
        if len(op.qubits) == 0 or len(op.qubits) > MAX_OP_QUBITS:
            raise ValueError(f"{op.name}: unsupported qubit count {len(op.qubits)}")
        if len(set(op.qubits)) != len(op.qubits):
            raise ValueError(f"{op.name}: repeated qubit in {op.qubits}")
        for q in op.qubits:
            if q < 0 or q >= num_qubits:
                raise ValueError(f"{op.name}: qubit {q} outside a {num_qubits}-qubit state")
        if op.kind == OP_MATRIX:
            k = len(op.qubits) - op.ncontrols
            if k < 1:
                raise ValueError(f"{op.name}: no target qubit")
            if op.matrix.shape != (1 << k, 1 << k):
                raise ValueError(f"{op.name}: matrix shape {op.matrix.shape} does not match {k} targets")
        for p in op.params:
            if not np.isfinite(p):
                raise ValueError(f"{op.name}: non-finite parameter {p}")


def pack(ops) -> tuple[np.ndarray, np.ndarray]:
    """Pack gate ops into (qfvm_op array, complex128 matrix pool)."""
    gates = [o for o in ops if o.is_gate and o.kind != OP_NOP]
    arr = np.zeros(len(gates), dtype=OP_DTYPE)
    pool = []
    off = 0
    for i, o in enumerate(gates):
        r = arr[i]
        r["kind"] = o.kind
        r["ncontrols"] = o.ncontrols
        r["nqubits"] = len(o.qubits)
        r["qubits"][: len(o.qubits)] = o.qubits
        r["slot"] = o.slot
        r["gen"] = o.gen
        p = list(o.params)[:4]
        r["params"][: len(p)] = p
        if o.matrix is not None:
            m = np.ascontiguousarray(o.matrix, dtype=np.complex128)
            r["mat_dim"] = m.shape[0]
            r["mat_offset"] = off
            pool.append(m.ravel())
            off += m.size
        else:
            r["mat_offset"] = -1
    pool_arr = np.concatenate(pool) if pool else np.zeros(1, dtype=np.complex128)
    return arr, np.ascontiguousarray(pool_arr, dtype=np.complex128)


def program_draws(ops) -> int:
    """Uniform draws one shot of a program consumes (one per measure / reset)."""
    return sum(1 for o in ops if o.kind in (OP_MEASURE, OP_RESET))


def pack_program(ops) -> tuple[np.ndarray, np.ndarray]:
    """Pack a whole program for qfvm_simulate_shots: gates as in ``pack``,
    measure (qubits, then classical bits at qubits[8:]), reset, and cif
    followed by its body (mat_dim = body length).  NOPs are dropped."""
    flat = []
    for o in ops:
        if o.kind == OP_NOP:
            continue
        if o.kind == OP_CIF:
            body = [b for b in o.body if b.kind != OP_NOP]
            if any(not b.is_gate for b in body):
                raise ValueError("a cif body holds gates only")
            flat.append(o)
            flat.extend(body)
        else:
            flat.append(o)
    gates_arr, pool = pack([o for o in flat if o.is_gate])
    arr = np.zeros(len(flat), dtype=OP_DTYPE)
    gi = 0
    for i, o in enumerate(flat):
        r = arr[i]
        if o.is_gate:
            arr[i] = gates_arr[gi]
            gi += 1
            continue
        r["kind"] = o.kind
        r["mat_offset"] = -1
        r["slot"] = -1
        if o.kind == OP_MEASURE:
            if len(o.qbits) > 8:
                raise ValueError("a measure of more than 8 qubits at once")
            r["nqubits"] = len(o.qbits)
            r["qubits"][: len(o.qbits)] = o.qbits
            r["qubits"][8: 8 + len(o.cbits)] = o.cbits
        elif o.kind == OP_RESET:
            if len(o.qbits) > 8:
                raise ValueError("a reset of more than 8 qubits at once")
            r["nqubits"] = len(o.qbits)
            r["qubits"][: len(o.qbits)] = o.qbits
        elif o.kind == OP_CIF:
            if len(o.cbits) > 16:
                raise ValueError("cif on more than 16 classical bits")
            r["nqubits"] = len(o.cbits)
            r["qubits"][: len(o.cbits)] = o.cbits
            r["params"][0] = float(o.condition)
            r["mat_dim"] = sum(1 for b in o.body if b.kind != OP_NOP)
    return arr, pool


# ------------------------------------------------------------------ noise


def channel_op(kind: int, qubit: int, matrices, probs=None) -> Op:
    """A one-qubit channel: ``matrices`` (m, 2, 2); unitary channels also
    carry the probabilities of their operators in ``params``."""
    mats = np.ascontiguousarray(np.asarray(matrices, dtype=np.complex128).reshape(-1, 2, 2))
    params = [] if probs is None else [float(p) for p in probs]
    name = "unitary_channel" if kind == OP_UCHANNEL else "kraus_channel"
    op = Op(name, kind, (qubit,), 0, (), matrix=mats)
    op.params = tuple(params)
    return op


def _is_instance_named(obj, names) -> bool:
    return any(c.__name__ in names for c in type(obj).__mro__)


def read_noisy_op(pyop) -> Op | None:
    """One instruction of a noisy circuit: UnitaryChannel (gatelist + probs,
    quafu/elements/noise.py:71-91) and KrausChannel (gatelist, :26-68) become
    channel ops; anything else is read as ``read_op`` does."""
    if _is_instance_named(pyop, ("UnitaryChannel", "KrausChannel")):
        mats = [_matrix_of(g) for g in pyop.gatelist]
        q = pyop.pos[0] if not isinstance(pyop.pos, (int, np.integer)) else int(pyop.pos)
        if _is_instance_named(pyop, ("UnitaryChannel",)):
            return channel_op(OP_UCHANNEL, int(q), mats, list(pyop.probs))
        return channel_op(OP_KRAUS, int(q), mats)
    return read_op(pyop)


def pack_noise(ops) -> tuple[np.ndarray, np.ndarray]:
    """Pack gates and channels for qfvm_simulate_noise: a channel's matrices
    (and, for unitary channels, its probabilities as the next m pool
    entries) go to the matrix pool."""
    gates_arr, gpool = pack([o for o in ops if o.is_gate])
    pool = [gpool] if any(o.is_gate and o.matrix is not None for o in ops) else []
    off = sum(p.size for p in pool)
    arr = np.zeros(len([o for o in ops if o.kind != OP_NOP]), dtype=OP_DTYPE)
    gi = 0
    i = 0
    for o in ops:
        if o.kind == OP_NOP:
            continue
        if o.is_gate:
            arr[i] = gates_arr[gi]
            gi += 1
        else:
            if o.kind not in (OP_UCHANNEL, OP_KRAUS):
                raise ValueError(f"'{o.name}' in a noisy circuit: gates and channels only")
            m = o.matrix.shape[0]
            r = arr[i]
            r["kind"] = o.kind
            r["nqubits"] = 1
            r["qubits"][0] = o.qubits[0]
            r["params"][0] = m
            r["mat_dim"] = 2
            r["mat_offset"] = off
            r["slot"] = -1
            block = [o.matrix.reshape(-1)]
            if o.kind == OP_UCHANNEL:
                block.append(np.asarray(o.params, dtype=np.complex128))
            block = np.concatenate(block)
            pool.append(block)
            off += block.size
        i += 1
    pool_arr = np.concatenate(pool) if pool else np.zeros(1, dtype=np.complex128)
    return arr, np.ascontiguousarray(pool_arr, dtype=np.complex128)


def noise_draws(ops) -> int:
    """Uniforms one noisy shot consumes: one per channel, one for the sample."""
    return sum(1 for o in ops if o.kind in (OP_UCHANNEL, OP_KRAUS)) + 1
