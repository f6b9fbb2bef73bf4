"""Adjoint gradients on the GPU against the reference's gradients (golden),
the oracle's restated adjoint, central finite differences (h = 1e-6) and the
GPU parameter-shift path.  Tolerances: complex128 and double-single 1e-10;
complex64 1e-5 (the accuracy bound for the batched complex64 path)."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import gradients, ir, workloads

pytestmark = pytest.mark.gpu


def assemble(assembly, gate_grads):
    return [sum(c * gate_grads[i] for i, c in row) for row in assembly]


def fd_oracle(n, ops, terms, h=1e-6):
    nslot = max(o.slot for o in ops) + 1
    base = [0.0] * nslot
    for o in ops:
        if o.slot >= 0:
            base[o.slot] = o.params[0]
    g = np.zeros(nslot)
    for k in range(nslot):
        vals = []
        for s in (h, -h):
            p = list(base)
            p[k] += s
            vals.append(oracle.energy(n, gradients.bind(ops, p), terms))
        g[k] = (vals[0] - vals[1]) / (2 * h)
    return g


@pytest.mark.parametrize("precision,tol", [("c128", 1e-10), ("c128_ds", 1e-10), ("c64", 1e-5)])
def test_golden_gradients(golden, precision, tol):
    meta, _ = golden
    for case in meta["gradients"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        terms = [(c, p, pos) for c, p, pos in case["terms"]]
        e, gg = gradients.adjoint(case["n"], ops, terms, precision, n_slots=len(ops))
        assert abs(e - case["energy"]) < tol
        np.testing.assert_allclose(assemble(case["assembly"], gg), case["adjoint"], atol=tol)


def test_param_shift_matches_reference(golden):
    meta, _ = golden
    for case in meta["gradients"]:
        if case["tag"] == "ref_test_gradient":
            continue  # its ParameterExpression gate is not a plain rotation slot
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        terms = [(c, p, pos) for c, p, pos in case["terms"]]
        ps = gradients.param_shift(case["n"], ops, terms, "c128")
        gg = np.zeros(len(ops))
        gg[: ps.size] = ps
        np.testing.assert_allclose(assemble(case["assembly"], gg), case["param_shift"], atol=1e-10)


@pytest.mark.parametrize("n", [6, 12, 14])
@pytest.mark.parametrize("precision,tol", [("c128", 1e-10), ("c128_ds", 1e-10), ("c64", 1e-5)])
def test_hea_matches_oracle_adjoint(n, precision, tol):
    ops, _ = workloads.hea(n, 4, seed=n)
    terms = workloads.zz_x_hamiltonian(n, seed=n)
    slots = [o.slot for o in ops]
    ref = oracle.grad_adjoint(n, ops, slots, terms)
    e, g = gradients.adjoint(n, ops, terms, precision)
    assert abs(e - oracle.energy(n, ops, terms)) < tol
    np.testing.assert_allclose(g, ref, atol=tol)


def test_all_generators_against_finite_differences():
    n = 12
    rng = np.random.default_rng(3)
    ops = [workloads.named("h", (q,)) for q in range(n)]
    slot = 0

    def add(op):
        nonlocal slot
        op.slot = slot
        slot += 1
        ops.append(op)

    for layer in range(2):
        for q in range(n):
            add(ir.Op("rx", ir.OP_RX, (q,), 0, (float(rng.uniform(0, 6)),)))
            add(ir.Op("ry", ir.OP_RY, ((q + 3) % n,), 0, (float(rng.uniform(0, 6)),)))
        add(ir.Op("rz", ir.OP_RZ, (5,), 0, (0.7,)))
        add(ir.Op("rzz", ir.OP_RZZ, (2, 9), 0, (1.3,)))
        add(ir.Op("p", ir.OP_P, (11,), 0, (0.4,)))
        add(ir.Op("cp", ir.OP_CP, (0, 7), 1, (2.2,)))
        for name, mat_fn, qs, nc in [
            ("crx", lambda t: np.array([[np.cos(t / 2), -1j * np.sin(t / 2)], [-1j * np.sin(t / 2), np.cos(t / 2)]]), (1, 6), 1),
            ("cry", lambda t: np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]]), (10, 4), 1),
            ("crz", lambda t: np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)]), (3, 8), 1),
        ]:
            t = float(rng.uniform(0, 6))
            op = ir.Op(name, ir.OP_MATRIX, qs, nc, (t,), matrix=mat_fn(t))
            add(op)
        for q in range(n - 1):
            ops.append(workloads.named("cx", (q, q + 1), ncontrols=1))
    terms = workloads.zz_x_hamiltonian(n, seed=1) + [(0.3, "Y", [4]), (0.2, "XY", [0, 5])]
    # matrix gates: rebuild their matrices from the (possibly shifted) angle
    mats = {"crx": lambda t: np.array([[np.cos(t / 2), -1j * np.sin(t / 2)], [-1j * np.sin(t / 2), np.cos(t / 2)]]),
            "cry": lambda t: np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]]),
            "crz": lambda t: np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])}

    def bound(params):
        out = []
        for o in ops:
            if o.slot >= 0 and o.matrix is not None:
                t = params[o.slot]
                out.append(ir.Op(o.name, o.kind, o.qubits, o.ncontrols, (t,), matrix=mats[o.name](t), slot=o.slot))
            elif o.slot >= 0:
                out.append(ir.Op(o.name, o.kind, o.qubits, o.ncontrols, (params[o.slot],), slot=o.slot))
            else:
                out.append(o)
        return out

    base = np.zeros(slot)
    for o in ops:
        if o.slot >= 0:
            base[o.slot] = o.params[0]
    fd = np.zeros(slot)
    h = 1e-6
    for k in range(slot):
        p1, p2 = base.copy(), base.copy()
        p1[k] += h
        p2[k] -= h
        fd[k] = (oracle.energy(n, bound(p1), terms) - oracle.energy(n, bound(p2), terms)) / (2 * h)
    _, g = gradients.adjoint(n, ops, terms, "c128")
    np.testing.assert_allclose(g, fd, atol=2e-8)


def test_many_probes_span_passes():
    # more parameterised gates than one pass holds probes for
    n = 14
    ops, _ = workloads.hea(n, 8, seed=2)
    terms = workloads.zz_x_hamiltonian(n, seed=2)
    ref = oracle.grad_adjoint(n, ops, [o.slot for o in ops], terms)
    _, g = gradients.adjoint(n, ops, terms, "c128")
    np.testing.assert_allclose(g, ref, atol=1e-10)


def test_input_state_gradient():
    n = 11
    ops, _ = workloads.hea(n, 3, seed=5)
    terms = workloads.zz_x_hamiltonian(n, seed=5)
    psi = helpers.random_state(n, 8)
    ref = oracle.grad_adjoint(n, ops, [o.slot for o in ops], terms, psi_in=psi)
    _, g = gradients.adjoint(n, ops, terms, "c128", psi=psi)
    np.testing.assert_allclose(g, ref, atol=1e-10)
