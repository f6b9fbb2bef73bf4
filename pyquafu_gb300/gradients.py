"""Gradients on the GB300 engine.

* ``adjoint``: energy and dE/dtheta for every parameter slot in one forward
  pass plus one reverse sweep over two device states (the method of
  quafu/algorithms/gradients/gradiant.py:144-173, fused on the GPU).
* ``param_shift``: (E(theta + pi/2) - E(theta - pi/2)) / 2 per parameterised
  rotation (gradiant.py:38-73), each energy a full GPU forward simulation;
  the baseline the adjoint method is compared with on the same GPU.
* ``grad_adjoint`` / ``grad_para_shift``: drop-ins for pyquafu's functions of
  the same names (same arguments, same chain rule through
  ``QuantumCircuit._calc_parameter_grads``).

Observables are lists of ``(coeff, paulistr, pos)`` terms.
"""

from __future__ import annotations

import numpy as np

from . import _native as nat
from . import ir
from .engine import DeviceState, Plan, _precision, pack_terms


def bind(ops, params):
    """Copy of ``ops`` whose slotted rotation angles are params[slot]."""
    out = []
    for o in ops:
        if o.slot >= 0 and o.matrix is None:
            p = list(o.params)
            p[0] = float(params[o.slot])
            o = ir.Op(o.name, o.kind, o.qubits, o.ncontrols, p, slot=o.slot, gen=o.gen)
        out.append(o)
    return out


def _terms_arrays(terms):
    x, z, y = pack_terms([(p, pos) for _, p, pos in terms])
    c = np.array([float(np.real(t[0])) for t in terms], dtype=np.float64)
    return x, z, y, c


def adjoint(n: int, ops, terms, precision="c128", psi=None, n_slots: int | None = None):
    """Returns (energy, grads[n_slots]) for E = sum_t c_t <psi|P_t|psi>."""
    lib = nat.load()
    gates = [o for o in ops if o.is_gate]
    if n_slots is None:
        n_slots = max([o.slot for o in gates] + [-1]) + 1
    arr, pool = ir.pack(gates)
    x, z, y, c = _terms_arrays(terms)
    grads = np.zeros(max(n_slots, 1), dtype=np.float64)
    energy = np.zeros(1, dtype=np.float64)
    psi_p = None
    if psi is not None:
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        psi_p = nat.dptr(psi.view(np.float64))
    rc = lib.qfvm_adjoint(n, _precision(precision), nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                          pool.size, nat.u64ptr(x), nat.u64ptr(z), nat.i32ptr(y), nat.dptr(c), c.size, psi_p,
                          nat.dptr(energy), nat.dptr(grads), n_slots)
    nat.check(rc, "adjoint")
    return float(energy[0]), grads[:n_slots]


def energy(n: int, ops, terms, precision="c128", state: DeviceState | None = None) -> float:
    """sum_t c_t <P_t> after running ``ops`` from |0..0> on the GPU."""
    own = state is None
    st = DeviceState(n, precision) if own else state
    st.set_zero()
    st.apply([o for o in ops if o.is_gate])
    vals = st.expect([(p, pos) for _, p, pos in terms])
    if own:
        st.close()
    return float(sum(float(np.real(t[0])) * v for t, v in zip(terms, vals)))


def param_shift(n: int, ops, terms, precision="c128"):
    """Parameter-shift gradient on the plain GPU path: two full simulations
    per parameterised rotation (rx, ry, rz, rzz and their matrix forms)."""
    gates = [o for o in ops if o.is_gate]
    n_slots = max([o.slot for o in gates] + [-1]) + 1
    grads = np.zeros(n_slots)
    st = DeviceState(n, precision)
    for i, o in enumerate(gates):
        if o.slot < 0:
            continue
        if o.matrix is not None:
            raise ValueError("parameter shift needs named rotation gates")
        res = []
        for sh in (np.pi / 2, -np.pi / 2):
            shifted = list(gates)
            p = list(o.params)
            p[0] += sh
            shifted[i] = ir.Op(o.name, o.kind, o.qubits, o.ncontrols, p, slot=o.slot)
            res.append(energy(n, shifted, terms, precision, st))
        grads[o.slot] += (res[0] - res[1]) / 2.0
    st.close()
    return grads


# ------------------------------ pyquafu drop-ins ------------------------------


def _circuit_terms(hamiltonian):
    return [(complex(p.coeff).real, p.paulistr, list(p.pos)) for p in hamiltonian.paulis]


def _slotted_ops(qc):
    """IR ops of ``qc`` with slot = index in qc.gates for gates whose first
    parameter is a pyquafu Parameter / ParameterExpression."""
    circ = ir.read_circuit(qc)
    gates = [o for o in circ.ops if o.is_gate]
    if len(gates) != len(qc.gates):
        raise ValueError("circuits with wrapped sub-circuits are not supported here: unwrap them first")
    for i, g in enumerate(qc.gates):
        paras = getattr(g, "paras", [])
        if paras and type(paras[0]).__name__ in ("Parameter", "ParameterExpression"):
            gates[i].slot = i
    return circ.num_qubits, gates, len(qc.gates)


def _assemble(para_grads, gate_grads):
    """assemble_grads (gradiant.py:24-35) over per-gate gradients."""
    out = []
    for var in para_grads:
        full = 0.0
        for pos, gp in para_grads[var]:
            full += gate_grads[pos[0]] * gp
        out.append(full)
    return out


def grad_adjoint(qc, hamiltonian, psi_in=np.array([], dtype=complex), precision="c128_ds"):
    """Drop-in for quafu.algorithms.gradients.grad_adjoint on the GPU
    (complex128 with float-pair arithmetic by default, as the engine's other
    complex128 work; "c128" for IEEE FP64)."""
    para_grads = qc._calc_parameter_grads()
    n, gates, ngates = _slotted_ops(qc)
    psi = None if psi_in is None or np.size(psi_in) == 0 else np.asarray(psi_in, dtype=np.complex128)
    _, gate_grads = adjoint(n, gates, _circuit_terms(hamiltonian), precision, psi, n_slots=ngates)
    return _assemble(para_grads, gate_grads)


def grad_para_shift(qc, hamiltonian, precision="c128_ds"):
    """Drop-in for quafu.algorithms.gradients.grad_para_shift on the GPU
    (float-pair complex128 by default)."""
    para_grads = qc._calc_parameter_grads()
    n, gates, _ = _slotted_ops(qc)
    return _assemble(para_grads, param_shift(n, gates, _circuit_terms(hamiltonian), precision))


# ---------------------------- batched parameter shift ----------------------------


def jacobian_param_shift(n: int, ops, observables, values, precision="c64", chunk_items: int = 8192):
    """The reference's parameter-shift Jacobian (ParamShift.grad,
    param_shift.py:47-78, looped over samples and observables in vjp.py:60-103)
    on the batched engine: every shifted evaluation (value[s] +- pi/2, one slot
    at a time) is one item of a batch run, and all observables of an item come
    from the same run.  values: (batch, slots).  Returns (expectation values
    (batch, n_obs), Jacobian (batch, n_obs, slots))."""
    from .batch import BatchSession

    values = np.atleast_2d(np.asarray(values, dtype=np.float64))
    b, s = values.shape
    gates = [o for o in ops if o.is_gate]
    # per sample: the unshifted point, then +pi/2 and -pi/2 on every slot
    shifts = np.concatenate([np.zeros((1, s)), np.eye(s) * (np.pi / 2), -np.eye(s) * (np.pi / 2)])
    per = shifts.shape[0]
    evals = (values[:, None, :] + shifts[None, :, :]).reshape(b * per, s)
    out = []
    sessions = {}
    try:
        for c0 in range(0, evals.shape[0], chunk_items):
            chunk = evals[c0: c0 + chunk_items]
            bs = sessions.get(chunk.shape[0])
            if bs is None:
                bs = BatchSession(precision, grads=False)
                bs.add_group(n, gates, observables, chunk.shape[0], s)
                sessions[chunk.shape[0]] = bs
            out.append(bs.run([chunk])[0])
    finally:
        for bs in sessions.values():
            bs.close()
    e = np.concatenate(out).reshape(b, per, -1)
    expv = e[:, 0, :]
    jac = (e[:, 1: 1 + s, :] - e[:, 1 + s:, :]) / 2.0  # (batch, slots, n_obs)
    return expv, np.transpose(jac, (0, 2, 1))
