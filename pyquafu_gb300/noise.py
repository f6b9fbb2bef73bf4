"""Noisy trajectories on the GB300 engine.

``NoiseSVSimulator`` mirrors quafu.simulators.simulator.NoiseSVSimulator
(simulator.py:148-225): every shot samples the circuit's unitary channels
(gen_circuit), runs it with its Kraus channels resolved one at a time
(_apply_op, :61-76), samples one outcome of the measured qubits and, with a
Hamiltonian, evaluates every term.  The reference runs the shots one after
another in Python; here all shots run side by side on the device through one
call (``qfvm_simulate_noise``).  Its draws come from numpy's global generator
and the engine's random device; here they are uniforms from a seeded host
generator (``qfvm.set_seed``) or given explicitly, in the reference's order:
unitary channels, then Kraus channels, then the sample.
"""

from __future__ import annotations

import numpy as np

from . import _native as nat
from . import ir
from . import qfvm
from .engine import pack_terms


def _noisy_ops(qc):
    ops = []

    def walk(instructions):
        for ins in instructions:
            if hasattr(ins, "circuit"):  # wrapped sub-circuit
                walk(ins.circuit.instructions)
                continue
            o = ir.read_noisy_op(ins)
            if o is None or o.kind in (ir.OP_MEASURE, ir.OP_NOP):
                continue
            if not (o.is_gate or o.kind in (ir.OP_UCHANNEL, ir.OP_KRAUS)):
                raise qfvm.QfvmError(f"'{o.name}' is not supported in a noisy circuit", 4)
            ops.append(o)

    walk(qc.instructions)
    return ops


def simulate_noise(n: int, ops, shots: int, psi=None, terms=None, uniforms=None):
    """Run ``shots`` noisy trajectories of the gate/channel list ``ops``.
    Returns (sampled basis index per shot, per-shot coeff * <P_t> array or
    None).  ``terms``: [(coeff, paulistr, pos)]; ``uniforms``: (shots,
    ir.noise_draws(ops)) or None for the seeded host generator."""
    shots = int(shots)
    if shots < 1:
        raise qfvm.QfvmError("noisy trajectories need shots >= 1", 1)
    for o in ops:
        if o.is_gate:
            ir.validate([o], n)
    nd = ir.noise_draws(ops)
    if uniforms is None:
        uniforms = qfvm._uniforms(shots * nd).reshape(shots, nd)
    uni = np.ascontiguousarray(uniforms, dtype=np.float64)
    if uni.shape != (shots, nd):
        raise ValueError(f"uniforms must have shape {(shots, nd)}")
    arr, pool = ir.pack_noise(ops)
    samples = np.zeros(shots, dtype=np.uint64)
    nt = len(terms) if terms else 0
    if nt:
        x, z, y = pack_terms([(p, pos) for _, p, pos in terms])
        c = np.array([float(np.real(t[0])) for t in terms], dtype=np.float64)
        ev = np.zeros(shots * nt)
    else:
        x = z = np.zeros(1, dtype=np.uint64)
        y = np.zeros(1, dtype=np.int32)
        c = ev = np.zeros(1)
    psi_p = None
    if psi is not None and np.size(psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        if psi.size != 1 << n:
            raise ValueError("input state does not match the circuit's qubit count")
        psi_p = nat.dptr(psi.view(np.float64))
    rc = nat.load().qfvm_simulate_noise(n, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)), pool.size,
                                        psi_p, shots, nat.dptr(uni), nd, nat.u64ptr(samples), nat.u64ptr(x),
                                        nat.u64ptr(z), nat.i32ptr(y), nat.dptr(c), nt, nat.dptr(ev))
    nat.check(rc, "noisy trajectories")
    return samples, (ev.reshape(shots, nt) if nt else None)


class NoiseSVSimulator:
    """Drop-in for quafu.simulators.simulator.NoiseSVSimulator."""

    def __init__(self, use_gpu: bool = False, use_custatevec: bool = False):
        self.use_gpu = use_gpu
        self.use_custatevec = use_custatevec

    def run(self, qc, psi=None, shots: int = 0, hamiltonian=None, uniforms=None):
        """Same result fields as the reference: counts {bitstring: count},
        pauli_expects (per term, averaged over shots), qbitnum, measures,
        simulator.  Returns quafu's SimuResult when quafu is importable."""
        ops = _noisy_ops(qc)
        terms = None
        if hamiltonian is not None:
            terms = [(complex(p.coeff).real, p.paulistr, list(p.pos)) for p in hamiltonian.paulis]
        samples, expv = simulate_noise(qc.num, ops, shots, psi, terms, uniforms)
        measures = list(dict(qc.measures).items())
        counts: dict = {}
        if measures:
            for st in qfvm._bitstrings(samples, measures):
                counts[st] = counts.get(st, 0) + 1
        pauli_expects = list(expv.mean(axis=0)) if expv is not None else []
        res_info = {"counts": counts, "pauli_expects": pauli_expects, "qbitnum": qc.num,
                    "measures": qc.measures, "simulator": "noisy statevector"}
        try:
            from quafu.results.results import SimuResult  # pylint: disable=import-outside-toplevel

            return SimuResult(res_info)
        except ImportError:
            return res_info
