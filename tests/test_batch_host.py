"""Batched plans on the CPU (no GPU): the pool blocks a batched run rewrites
per item (bind records) reproduce the planner's own coefficients, and a
batched plan interpreted with per-item rebound pools matches the oracle for
every item, forward (states) and reverse (adjoint gradients)."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import gradients, ir, workloads

named = workloads.named


def bind_coef(kind, th):
    """Coefficients of a bindable gate at angle th, as the planner lays them out."""
    c, s = np.cos(th / 2), np.sin(th / 2)
    if kind == ir.OP_RX:
        return [c, s]
    if kind == ir.OP_RY:
        return [c, -s, s, c]
    if kind in (ir.OP_RZ, ir.OP_RZZ):
        return [c, -s, c, s]
    if kind in (ir.OP_P, ir.OP_CP):
        return [1.0, 0.0, np.cos(th), np.sin(th)]
    raise AssertionError(kind)


def rebind(plan, values):
    coef = plan["coef"].copy()
    for off, kind, sign, slot in plan["binds"]:
        c = bind_coef(int(kind), float(sign) * float(values[slot]))
        coef[off: off + len(c)] = c
    return dict(plan, coef=coef)


def mixed_circuit(n, seed):
    """Slotted rx/ry/rz/p/cp/rzz with template angles at the special values
    (0, pi, pi/2) that single-state plans specialise, plus fixed gates."""
    rng = np.random.default_rng(seed)
    ops, slot = [], 0
    special = [0.0, np.pi, np.pi / 2, -np.pi / 2]
    for layer in range(3):
        for q in range(n):
            ops.append(named("h" if (q + layer) % 3 == 0 else "t", (q,)))
        for q in range(n):
            name = ["rx", "ry", "rz", "p"][(q + layer) % 4]
            ops.append(ir.Op(name, ir.NAMED_KIND[name], (q,), 0, (special[(q + layer) % 4],), slot=slot))
            slot += 1
        for q in range(0, n - 1, 2):
            ops.append(ir.Op("cp", ir.OP_CP, (q, q + 1), 1, (special[layer % 4],), slot=slot))
            slot += 1
        for q in range(1, n - 1, 2):
            ops.append(ir.Op("rzz", ir.OP_RZZ, (q, q + 1), 0, (float(rng.uniform(0, 2 * np.pi)),), slot=slot))
            slot += 1
        for q in range(n - 1):
            ops.append(named("cx", (q, q + 1), ncontrols=1))
    return ops, slot


def template_values(ops, nslots):
    v = np.zeros(nslots)
    for o in ops:
        if o.slot >= 0:
            v[o.slot] = o.params[0]
    return v


@pytest.mark.parametrize("n,adjoint", [(5, False), (13, False), (5, True), (12, True)])
def test_binds_reproduce_planner_coefficients(n, adjoint):
    ops, nslots = mixed_circuit(n, seed=n)
    plan = helpers.host_plan(n, ops, precision=0, adjoint=adjoint, batched=True)
    nslotted = sum(1 for o in ops if o.slot >= 0)
    assert len(plan["binds"]) == nslotted  # one block per slotted gate (forward or its inverse)
    assert set(int(s) for s in plan["binds"][:, 2]) == {-1 if adjoint else 1}
    again = rebind(plan, template_values(ops, nslots))
    np.testing.assert_allclose(again["coef"], plan["coef"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("n", [5, 13])
def test_batched_forward_items_match_oracle(n):
    ops, nslots = mixed_circuit(n, seed=7 + n)
    plan = helpers.host_plan(n, ops, precision=0, batched=True)
    rng = np.random.default_rng(n)
    for item in range(3):
        v = rng.uniform(-np.pi, np.pi, nslots)
        if item == 0:
            v[::3] = np.pi  # values at which single-state plans would specialise
        psi = helpers.interpret(rebind(plan, v), oracle.zero_state(n))
        ref = oracle.simulate(n, gradients.bind(ops, v))
        assert np.max(np.abs(psi - ref)) < 1e-12


def _rot_only(n, layers, seed):
    enc = np.random.default_rng(seed).uniform(-np.pi, np.pi, n)
    return workloads.hea(n, layers, seed=seed, encode=enc)


@pytest.mark.parametrize("n", [6, 12])
def test_batched_adjoint_items_match_oracle(n):
    ops, params = _rot_only(n, 2, seed=n)
    nslots = max(o.slot for o in ops) + 1
    terms = [(1.0, "Z", [0]), (0.5, "XX", [0, 1])]
    rev = helpers.host_plan(n, ops, precision=0, adjoint=True, batched=True)
    fwd = helpers.host_plan(n, ops, precision=0, batched=True)
    rng = np.random.default_rng(3)
    for _ in range(2):
        v = rng.uniform(-np.pi, np.pi, nslots)
        psi = helpers.interpret(rebind(fwd, v), oracle.zero_state(n))
        lam = oracle.apply_hamiltonian(psi, terms)
        vals = helpers.interpret2(rebind(rev, v), psi, lam)
        g = np.zeros(nslots)
        for p, s in enumerate(rev["probe_slots"]):
            g[s] += vals[p]
        bound = gradients.bind(ops, v)
        ref = oracle.grad_adjoint(n, bound, [o.slot for o in bound], terms)
        np.testing.assert_allclose(g, ref, atol=1e-11)


def test_batched_adjoint_phase_gates_by_finite_differences():
    n = 5
    ops, nslots = mixed_circuit(n, seed=11)
    terms = [(1.0, "Z", [0]), (-0.7, "ZZ", [1, 2]), (0.3, "Y", [3])]
    rev = helpers.host_plan(n, ops, precision=0, adjoint=True, batched=True)
    fwd = helpers.host_plan(n, ops, precision=0, batched=True)
    v = np.random.default_rng(5).uniform(-np.pi, np.pi, nslots)
    psi = helpers.interpret(rebind(fwd, v), oracle.zero_state(n))
    vals = helpers.interpret2(rebind(rev, v), psi, oracle.apply_hamiltonian(psi, terms))
    g = np.zeros(nslots)
    for p, s in enumerate(rev["probe_slots"]):
        g[s] += vals[p]
    h = 1e-6
    fd = np.zeros(nslots)
    for k in range(nslots):
        e = []
        for sh in (h, -h):
            w = v.copy()
            w[k] += sh
            e.append(oracle.energy(n, gradients.bind(ops, w), terms))
        fd[k] = (e[0] - e[1]) / (2 * h)
    np.testing.assert_allclose(g, fd, atol=1e-7)


def test_unbindable_slot_is_rejected():
    from pyquafu_gb300 import _native as nat

    m = np.eye(2, dtype=np.complex128)
    ops = [ir.Op("u", ir.OP_MATRIX, (0,), 0, (0.3,), matrix=m, slot=0)]
    with pytest.raises(nat.QfvmError, match="per-item parameter"):
        helpers.host_plan(2, ops, batched=True)
