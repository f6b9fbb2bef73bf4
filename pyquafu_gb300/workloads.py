"""Seeded synthetic circuits for the benchmark configurations.

Random layered circuits (the statevector sweeps):
  each layer applies one gate from {h, x, s, t, rx, ry, rz} to every qubit
  (angles uniform in [0, 2*pi)), then cx on a random perfect matching of the
  qubits; with ``extras`` about 5% of the layers also get cz, swap and rzz
  (uniform angle) on random pairs and ccx on a random triple.

Hardware-efficient ansatz (the gradient workloads):
  ``layers`` x (ry on every qubit, rz on every qubit) followed by a cx ladder
  0->1->...->n-1, optionally preceded by an ry angle-encoding layer.

Batched gradient workloads:
  ``uneven_batch``: circuits with qubit counts uniform in [nmin, nmax], each
  an ry(x_j) encoding layer (x ~ U[-pi, pi]) then ``layers`` HEA layers with
  angles ~ U[0, 2*pi); grouped by qubit count for the batched engine.
  ``qnn_batch``: a QNN on n qubits with ``layers`` HEA layers of shared
  weights, inputs x ~ N(0, 1) angle-encoded by ry, labels sign(w . x) for a
  fixed random w; the loss is the MSE of <Z_0> against the labels.

Circuits are returned as ``pyquafu_gb300.ir.Op`` lists (the engine's packed
input), and ``as_protocol`` wraps them in objects with the attributes the
reference's circuit reader uses (.instructions, .num, .cbits_num; ops with
.name, .pos, ._paras, .ctrls, .matrix), so the drop-in ``qfvm`` module can be
exercised without pyquafu installed.
"""

from __future__ import annotations

import numpy as np

from . import ir

SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)
ONE_QUBIT = ("h", "x", "s", "t", "rx", "ry", "rz")


def named(name: str, qubits, params=(), ncontrols=0) -> ir.Op:
    return ir.Op(name, ir.NAMED_KIND[name], qubits, ncontrols, params)


def matrix_gate(name: str, qubits, matrix, ncontrols=0) -> ir.Op:
    return ir.Op(name, ir.OP_MATRIX, qubits, ncontrols, (), matrix=np.asarray(matrix, dtype=np.complex128))


def random_layers(n: int, depth: int, seed: int = 0, extras: bool = False, extra_rate: float = 0.05) -> list:
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(depth):
        for q in range(n):
            g = ONE_QUBIT[int(rng.integers(len(ONE_QUBIT)))]
            if g in ("rx", "ry", "rz"):
                ops.append(named(g, (q,), (float(rng.uniform(0.0, 2 * np.pi)),)))
            else:
                ops.append(named(g, (q,)))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            ops.append(named("cx", (int(perm[i]), int(perm[i + 1])), ncontrols=1))
        if extras and n >= 3 and rng.random() < extra_rate:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(named("cz", (a, b), ncontrols=1))
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(matrix_gate("swap", (a, b), SWAP))
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(named("rzz", (a, b), (float(rng.uniform(0.0, 2 * np.pi)),)))
            a, b, c = (int(x) for x in rng.choice(n, 3, replace=False))
            ops.append(named("ccx", (a, b, c), ncontrols=2))
    return ops


def hea(n: int, layers: int, seed: int = 0, encode: np.ndarray | None = None):
    """Hardware-efficient ansatz.  Returns (ops, params); every ry/rz of the
    ansatz carries a parameter slot (0..2*n*layers-1); encoding gates carry
    slots after those."""
    rng = np.random.default_rng(seed)
    nparam = 2 * n * layers
    params = rng.uniform(0.0, 2 * np.pi, nparam)
    ops = []
    if encode is not None:
        for q in range(n):
            ops.append(ir.Op("ry", ir.OP_RY, (q,), 0, (float(encode[q]),), slot=nparam + q))
    k = 0
    for _ in range(layers):
        for q in range(n):
            ops.append(ir.Op("ry", ir.OP_RY, (q,), 0, (float(params[k]),), slot=k))
            k += 1
        for q in range(n):
            ops.append(ir.Op("rz", ir.OP_RZ, (q,), 0, (float(params[k]),), slot=k))
            k += 1
        for q in range(n - 1):
            ops.append(named("cx", (q, q + 1), ncontrols=1))
    return ops, params


def uneven_batch(circuits: int = 2048, nmin: int = 10, nmax: int = 18, layers: int = 6, seed: int = 0):
    """Returns {n: (ops, values)} with values[item] the slot vector of one
    circuit: its 2 * n * layers HEA angles, then its n encoding angles."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, size=circuits)
    groups = {}
    for n in range(nmin, nmax + 1):
        count = int(np.sum(ns == n))
        if count == 0:
            continue
        ops, _ = hea(n, layers, seed=0, encode=np.zeros(n))
        nw = 2 * n * layers
        vals = np.empty((count, nw + n))
        vals[:, :nw] = rng.uniform(0.0, 2 * np.pi, (count, nw))
        vals[:, nw:] = rng.uniform(-np.pi, np.pi, (count, n))
        groups[n] = (ops, vals)
    return groups


def qnn_batch(batch: int = 1024, n: int = 16, layers: int = 12, seed: int = 0):
    """Returns (ops, weights, x, y): ops with slots 0..2*n*layers-1 for the
    shared weights and 2*n*layers + j for input feature j."""
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(batch, n))
    w = rng.normal(size=n)
    y = np.where(x @ w >= 0, 1.0, -1.0)
    ops, weights = hea(n, layers, seed=seed, encode=np.zeros(n))
    return ops, weights, x, y


def zz_x_hamiltonian(n: int, seed: int = 0):
    """sum_i a_i Z_i Z_{i+1} + sum_i b_i X_i with a, b ~ N(0, 1): list of
    (coeff, paulistr, pos)."""
    rng = np.random.default_rng(seed)
    a = rng.normal(size=n - 1)
    b = rng.normal(size=n)
    terms = [(float(a[i]), "ZZ", [i, i + 1]) for i in range(n - 1)]
    terms += [(float(b[i]), "X", [i]) for i in range(n)]
    return terms


# ------------------------- circuit-protocol wrappers -------------------------


class Parameter:
    """Stand-in with the reference Parameter's protocol (a named value that
    converts to float; quafu/elements/parameters.py:256-280)."""

    def __init__(self, name: str, value: float = 0.0):
        self.name = name
        self.value = float(value)

    def __float__(self):
        return self.value


class ParameterExpression:
    """Stand-in with the reference ParameterExpression's protocol
    (quafu/elements/parameters.py:24-107): ``_variables`` maps its
    Parameters to positions, ``_func(x)`` is its value at variable values x,
    ``grad(x)`` its gradient there.  Here built from a function and its
    gradient over the listed Parameters."""

    def __init__(self, variables, func, grad):
        self._vars = list(variables)
        self._f, self._g = func, grad

    @property
    def _variables(self):
        return {v: i for i, v in enumerate(self._vars)}

    @property
    def _func(self):
        return self._f

    def grad(self, input_value=None):
        if input_value is None or len(input_value) == 0:
            input_value = np.array([v.value for v in self._vars])
        return np.asarray(self._g(np.asarray(input_value, dtype=np.float64)))

    def __float__(self):
        return float(self._f(np.array([v.value for v in self._vars])))


class _ProtoGate:
    def __init__(self, op: ir.Op, variables=None):
        self.name = op.name.upper()
        self.pos = list(op.qubits)
        self._paras = list(op.params)
        if variables is not None and op.slot >= 0:
            self._paras[0] = variables[op.slot]
        self.paras = list(self._paras)
        if op.ncontrols:
            self.ctrls = list(op.qubits[: op.ncontrols])
        if op.matrix is not None:
            self.matrix = op.matrix


class _ProtoMeasure:
    name = "measure"

    def __init__(self, qbits, cbits):
        self.qbits = list(qbits)
        self.cbits = list(cbits)


class ProtoCircuit:
    """Minimal object with the circuit protocol the qfvm reader consumes."""

    def __init__(self, num: int, ops, measures=None, cbits_num=None, parameters: bool = False):
        self.num = num
        self.cbits_num = num if cbits_num is None else cbits_num
        # with ``parameters``, op slot k becomes the shared Parameter "theta_k"
        nslot = max([o.slot for o in ops] + [-1]) + 1
        self._vars = [Parameter(f"theta_{k}") for k in range(nslot)] if parameters else None
        if self._vars is not None:
            for o in ops:
                if o.slot >= 0:
                    self._vars[o.slot].value = o.params[0]
        self.instructions = [_ProtoGate(o, self._vars) for o in ops]
        self.gates = [g for g in self.instructions]
        if measures:
            q, c = zip(*measures)
            self.instructions.append(_ProtoMeasure(q, c))
        self.measures = dict(measures or [])

    def get_parameter_grads(self):
        """{Parameter: [[(gate index, para index), d angle / d parameter]]}
        in order of first use (quantum_circuit.py:255-283)."""
        out = {}
        for i, g in enumerate(self.gates):
            for j, p in enumerate(getattr(g, "paras", [])):
                if isinstance(p, Parameter):
                    out.setdefault(p, []).append([(i, j), 1.0])
                elif isinstance(p, ParameterExpression):
                    for v in p._variables:
                        out.setdefault(v, []).append([(i, j), 0.0])
        return out

    def _calc_parameter_grads(self):
        """quantum_circuit.py:285-297: d angle / d variable at the current
        values (expressions through their own grad)."""
        grads = self.get_parameter_grads()
        for var, items in grads.items():
            for item in items:
                i, j = item[0]
                p = self.gates[i].paras[j]
                if isinstance(p, ParameterExpression):
                    item[1] = float(p.grad()[p._variables[var]])
        return grads

    @property
    def variables(self):
        return list(self.get_parameter_grads().keys())


def as_protocol(num: int, ops, measures=None) -> ProtoCircuit:
    return ProtoCircuit(num, ops, measures)
