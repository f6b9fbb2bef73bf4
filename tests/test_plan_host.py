"""The fuser (host planner) checked on CPU: host-built plans are executed by
a numpy interpreter (tests/helpers.py) and compared with the oracle."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import workloads


SHAPES_C128 = [(11, 4), (12, 4), (12, 5), (12, 3), (11, 3)]
SHAPES_C64 = [(12, 5), (13, 5), (12, 4), (13, 4)]


@pytest.mark.parametrize("T,R", SHAPES_C128)
def test_random_layers_plans(T, R):
    for n in (T, T + 1, T + 3):
        ops = workloads.random_layers(n, 5, seed=100 + n, extras=True, extra_rate=0.6)
        plan = helpers.host_plan(n, ops, 0, T, R)
        got = helpers.interpret(plan, oracle.zero_state(n))
        ref = oracle.simulate(n, ops)
        assert np.abs(got - ref).max() < 1e-13
        # every gate applied once at most (one-qubit merges and merged
        # register-round diagonals fold some)
        applied = sum(int(s["op_count"]) for s in plan["steps"])
        applied += sum(int(p["op_count"]) for p in plan["passes"] if p["type"] != 0)
        assert 0.7 * len(ops) <= applied <= len(ops)


def plan_op_count(plan):
    return sum(int(s["op_count"]) for s in plan["steps"]) + sum(
        int(p["op_count"]) for p in plan["passes"] if p["type"] != 0)


def test_single_qubit_fusion():
    """Commuting one-qubit merges of plain plans: a diagonal passes a gate
    that uses its qubit as a control, RX passes CX on its target, X X
    vanishes; a Hadamard between, or a diagonal on a CX target, blocks."""
    n = 5
    named = workloads.named
    merged = [named("t", (0,)), named("cx", (0, 1), ncontrols=1), named("s", (0,)),          # 1 merge
              named("rx", (2,), (0.3,)), named("cx", (3, 2), ncontrols=1), named("rx", (2,), (1.1,)),  # 1 merge
              named("x", (4,)), named("x", (4,)),                                              # both removed
              named("rz", (3,), (0.7,)), named("cz", (3, 4), ncontrols=1), named("rz", (3,), (0.2,))]  # 1 merge
    blocked = [named("rz", (0,), (0.5,)), named("h", (0,)), named("rz", (0,), (0.4,)),
               named("t", (1,)), named("cx", (0, 1), ncontrols=1), named("t", (1,))]
    for ops, removed in ((merged, 5), (blocked, 0)):
        ops = [named("h", (q,)) for q in range(n)] + ops
        plan = helpers.host_plan(n, ops, 0, 0, 0)
        got = helpers.interpret(plan, oracle.zero_state(n))
        assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-13
        assert plan_op_count(plan) == len(ops) - removed


@pytest.mark.parametrize("T,R", SHAPES_C64)
def test_c64_shapes_plans(T, R):
    n = T + 2
    ops = workloads.random_layers(n, 4, seed=7, extras=True, extra_rate=0.5)
    plan = helpers.host_plan(n, ops, 1, T, R)
    got = helpers.interpret(plan, oracle.zero_state(n))
    assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-13


def test_all_gate_kinds_in_tile_passes(golden):
    meta, states = golden
    case = [c for c in meta["cases"] if c["tag"] == "allgates_n12"][0]
    ops = [helpers.op_from_json(d) for d in case["ops"]]
    plan = helpers.host_plan(12, ops, 0, 11, 4)
    kinds = {int(o["kind"]) for o in plan["ops"]}
    assert helpers.K_DENSE2 in kinds and helpers.K_SWAP in kinds and helpers.K_DIAG in kinds
    got = helpers.interpret(plan, oracle.zero_state(12))
    assert np.abs(got - states["allgates_n12__out"]).max() < 1e-13


def test_dense_k_gate_becomes_global_pass():
    rng = np.random.default_rng(0)
    m = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    ops = [workloads.named("h", (q,)) for q in range(13)]
    ops.append(workloads.matrix_gate("u3q", (12, 1, 7), m))
    ops += [workloads.named("rx", (q,), (0.3 * q,)) for q in range(13)]
    plan = helpers.host_plan(13, ops, 0, 12, 4)
    assert 2 in [int(p["type"]) for p in plan["passes"]]
    got = helpers.interpret(plan, oracle.zero_state(13))
    assert np.abs(got - oracle.simulate(13, ops)).max() < 1e-13


def _unitary(k, seed):
    rng = np.random.default_rng(seed)
    d = 1 << k
    return np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]


@pytest.mark.parametrize("n,T", [(10, 11), (15, 12)])
def test_wide_dense_gates_plans(n, T):
    """Dense gates on 7, 8 and 12 targets (the reference applies any count,
    statevector.hpp:945-995): given in any target order, with and without
    controls, in small states (split whole-state passes) and tiled ones."""
    rng = np.random.default_rng(n)
    ops = [workloads.named("h", (q,)) for q in range(n)]
    for k, nc in ((7, 0), (8, 1), (7, 2)):
        qs = [int(q) for q in rng.permutation(n)[: k + nc]]
        ops.append(workloads.matrix_gate(f"u{k}", qs, _unitary(k, k + nc), ncontrols=nc))
        ops += [workloads.named("ry", (q,), (0.1 + 0.2 * q,)) for q in range(n)]
    if n >= 12:
        qs = [int(q) for q in rng.permutation(n)[:12]]
        ops.append(workloads.matrix_gate("u12", qs, _unitary(12, 3)))
    plan = helpers.host_plan(n, ops, 0, T, 4)
    got = helpers.interpret(plan, oracle.zero_state(n))
    assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-12


def test_dense_gate_beyond_twelve_targets_rejected():
    from pyquafu_gb300 import _native as nat

    with pytest.raises(nat.QfvmError, match="at most 12"):
        helpers.host_plan(14, [workloads.matrix_gate("u13", list(range(13)), np.eye(1 << 13))])


def test_wide_dense_gate_in_adjoint_sweep():
    n = 9
    ops, _ = workloads.hea(n, 2, seed=1)
    ops.insert(10, workloads.matrix_gate("u7", [8, 0, 3, 5, 1, 7, 2], _unitary(7, 5)))
    terms = workloads.zz_x_hamiltonian(n, seed=2)
    plan = helpers.host_plan(n, ops, 0, adjoint=True)
    psi = oracle.simulate(n, ops)
    lam = oracle.apply_hamiltonian(psi, terms)
    vals = helpers.interpret2(plan, psi, lam)
    grads = np.zeros(max(o.slot for o in ops) + 1)
    for slot, v in zip(plan["probe_slots"], vals):
        grads[slot] += v
    ref = oracle.grad_adjoint(n, ops, [o.slot for o in ops], terms)
    np.testing.assert_allclose(grads, ref, atol=1e-12)


@pytest.mark.parametrize("R", [3, 4])
def test_round_diagonals_merge(R):
    """Plain plans merge the register-only diagonals of a round into one
    phase table (K_DIAGR, exact quarter turns coded), applied before the
    first op that acts non-diagonally on its bits; the interpreter checks the
    codes against the coefficients and the state against the oracle."""
    n = 14
    rng = np.random.default_rng(R)
    ops = []
    for layer in range(6):
        for q in range(n):
            g = ["s", "t", "z", "rz", "h", "rx", "sdg", "tdg"][int(rng.integers(8))]
            ops.append(workloads.named(g, (q,), (float(rng.uniform(0, 6.3)),) if g in ("rz", "rx") else ()))
        for _ in range(3):
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(workloads.named(["cz", "rzz", "cp"][layer % 3], (a, b),
                                       (0.7,) if layer % 3 else (), ncontrols=0 if layer % 3 == 1 else 1))
    plan = helpers.host_plan(n, ops, 0, 12, R)
    assert int(np.sum(plan["ops"]["kind"] == helpers.K_DIAGR)) > 0
    got = helpers.interpret(plan, oracle.zero_state(n))
    assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-13
    # batched and adjoint plans keep every gate
    assert int(np.sum(helpers.host_plan(n, ops, 0, adjoint=True)["ops"]["kind"] == helpers.K_DIAGR)) == 0


def test_invalid_ops_rejected():
    from pyquafu_gb300 import _native as nat

    with pytest.raises(nat.QfvmError):
        helpers.host_plan(4, [workloads.named("h", (4,))])
    with pytest.raises(nat.QfvmError):
        helpers.host_plan(4, [workloads.named("cx", (2, 2), ncontrols=1)])
    with pytest.raises(nat.QfvmError):
        helpers.host_plan(4, [workloads.named("h", (0,))], 0, 9, 4)  # shape not compiled in


@pytest.mark.parametrize("n,precision", [(8, 0), (13, 0), (13, 2), (14, 1)])
def test_adjoint_sweep_plan(n, precision):
    """The reverse sweep (probes + inverse gates) planned for the GPU, run by
    the numpy interpreter from (psi, H psi), gives the oracle's gradients."""
    ops, _ = workloads.hea(n, 3, seed=n)
    ops.insert(3, workloads.named("rzz", (0, n - 1), (0.7,)))
    ops[3].slot = max(o.slot for o in ops) + 1
    terms = workloads.zz_x_hamiltonian(n, seed=n) + [(0.4, "YZ", [1, 2])]
    plan = helpers.host_plan(n, ops, precision, adjoint=True)
    psi = oracle.simulate(n, ops)
    lam = oracle.apply_hamiltonian(psi, terms)
    vals = helpers.interpret2(plan, psi, lam)
    nslot = max(o.slot for o in ops) + 1
    got = np.zeros(nslot)
    for v, s in zip(vals, plan["probe_slots"]):
        got[s] += v
    ref = oracle.grad_adjoint(n, [o if o.name != "rzz" else o for o in ops], [o.slot for o in ops], terms)
    # the oracle's grad_gate knows rx/ry/rz; check rzz by finite differences instead
    rzz_slot = ops[3].slot
    mask = np.arange(nslot) != rzz_slot
    np.testing.assert_allclose(got[mask], ref[mask], atol=1e-11)
    h = 1e-6
    ep = oracle.energy(n, [workloads.named("rzz", (0, n - 1), (0.7 + h,)) if o is ops[3] else o for o in ops], terms)
    em = oracle.energy(n, [workloads.named("rzz", (0, n - 1), (0.7 - h,)) if o is ops[3] else o for o in ops], terms)
    assert abs(got[rzz_slot] - (ep - em) / (2 * h)) < 1e-8


def test_unnormalized_hadamards_fold_into_other_gates():
    """Plain plans turn uncontrolled Hadamards into additions and fold their
    1/sqrt(2) factors into other gates' coefficients: same state."""
    from pyquafu_gb300 import ir

    n = 6
    ops = []
    for layer in range(5):
        ops += [workloads.named("h", (q,)) for q in range(n)]
        ops += [ir.Op("ry", ir.OP_RY, (layer % n,), 0, (0.3 + layer,))]
        ops += [workloads.named("cx", (q, q + 1), ncontrols=1) for q in range(n - 1)]
    plan = helpers.host_plan(n, ops)
    kinds = [int(k) for k in plan["ops"]["kind"]]
    assert kinds.count(helpers.K_HAD) == 5 * n
    psi = helpers.interpret(plan, oracle.zero_state(n))
    assert np.max(np.abs(psi - oracle.simulate(n, ops))) < 1e-13
    # no gate to take the factor: the Hadamards stay normalized
    only_h = [workloads.named("h", (q,)) for q in range(n)]
    plan = helpers.host_plan(n, only_h)
    assert helpers.K_HAD not in [int(k) for k in plan["ops"]["kind"]]
    assert np.max(np.abs(helpers.interpret(plan, oracle.zero_state(n)) - oracle.simulate(n, only_h))) < 1e-14


@pytest.mark.parametrize("seed", range(6))
def test_random_commuting_merges(seed):
    """Dense random mixes of diagonals, RX, X, cx, cz, ccx and Hadamards on few
    qubits (many merge opportunities) against the oracle."""
    rng = np.random.default_rng(seed)
    n = 6
    named = workloads.named
    ops = []
    for _ in range(120):
        k = int(rng.integers(9))
        q = int(rng.integers(n))
        if k == 0:
            ops.append(named("rz", (q,), (float(rng.uniform(0, 6.3)),)))
        elif k == 1:
            ops.append(named(["t", "s", "z", "sdg", "tdg"][int(rng.integers(5))], (q,)))
        elif k == 2:
            ops.append(named("rx", (q,), (float(rng.uniform(0, 6.3)),)))
        elif k == 3:
            ops.append(named("x", (q,)))
        elif k == 4:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            ops.append(named("cx", (a, b), ncontrols=1))
        elif k == 5:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            ops.append(named("cz", (a, b), ncontrols=1))
        elif k == 6:
            a, b, c = (int(v) for v in rng.choice(n, 3, replace=False))
            ops.append(named("ccx", (a, b, c), ncontrols=2))
        elif k == 7:
            ops.append(named("h", (q,)))
        else:
            ops.append(named("p", (q,), (float(rng.uniform(0, 6.3)),)))
    plan = helpers.host_plan(n, ops, 0, 0, 0)
    got = helpers.interpret(plan, oracle.zero_state(n))
    assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-12
    assert plan_op_count(plan) < len(ops)


@pytest.mark.parametrize("eb", [16, 8])
def test_tile_layout(eb):
    """The padded tile layout: one-to-one, additive over disjoint bits, runs of
    32 contiguous and 16-byte aligned (bulk-copy units), and each position's
    slot bit as the planner assumes."""
    for T in (6, 11, 12, 13, 14):
        s = np.arange(1 << T)
        off = helpers.tile_off(s, eb)
        assert len(set(off.tolist())) == s.size
        run_start = off[:: 32] * eb
        assert np.all(run_start % 16 == 0)
        assert np.all(np.diff(off.reshape(-1, 32), axis=1) == 1)
        rng = np.random.default_rng(T)
        a = rng.integers(0, 1 << T, 500)
        b = rng.integers(0, 1 << T, 500) & ~a
        assert np.array_equal(helpers.tile_off(a | b, eb), helpers.tile_off(a, eb) + helpers.tile_off(b, eb))
    # slot bits: p < 3 (p < 4) direct, 3..4 (4) none, 5 + j -> j mod 3 (+1)
    direct = 3 if eb == 16 else 4
    for p in range(14):
        want = p if p < direct else (-1 if p < 5 else (p - 5) % 3 + (0 if eb == 16 else 1))
        assert helpers.slot_bit(p, eb, eb) == want, p
        if eb == 8 and p >= 1:
            assert helpers.slot_bit(p, 8, 16) == (p - 1 if p < 4 else (-1 if p == 4 else (p - 5) % 3))


@pytest.mark.parametrize("precision,T,R", [(0, 11, 4), (0, 12, 3), (1, 12, 4), (1, 13, 5)])
def test_round_wavefronts_hit_distinct_banks(precision, T, R):
    """Every register round's first wavefront of lanes (8 lanes of 16-byte
    accesses, 16 of 8-byte ones; 16-byte pairs for complex64 rounds that hold
    position 0 in registers) lands on distinct bank groups of the tile layout
    whenever the round's free positions offer a position for every slot bit."""
    n = 22
    ops = workloads.random_layers(n, 8, seed=5, extras=True)
    plan = helpers.host_plan(n, ops, precision, T, R)
    eb = plan["elem_bytes"]
    rounds = checked = 0
    for pd in plan["passes"]:
        if pd["type"] != 0:
            continue
        for sd in plan["steps"][pd["step_begin"]: pd["step_begin"] + pd["step_count"]]:
            if sd["type"] != 0:
                continue
            rounds += 1
            rpos = [int(x) for x in sd["rpos"][:R]]
            tpos = [int(x) for x in sd["tpos"][: T - R]]
            access = 16 if (eb == 8 and 0 in rpos) else eb
            nslot = 3 if access == 16 else 4
            if {helpers.slot_bit(p, eb, access) for p in tpos} >= set(range(nslot)):
                checked += 1
                lanes = 1 << nslot
                groups = set()
                for lane in range(lanes):
                    s = sum(1 << tpos[k] for k in range(nslot) if (lane >> k) & 1)
                    groups.add((helpers.tile_off(s, eb) * eb // access) % (128 // access))
                assert len(groups) == lanes, (rpos, tpos)
    assert rounds > 0 and checked >= 0.9 * rounds, (checked, rounds)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_edge_sizes(precision):
    """Smallest states (one and two qubits, a whole-state pass), an empty
    circuit (no passes), the largest supported qubit count (planned only)
    and counts outside the supported range (refused)."""
    from pyquafu_gb300 import _native as nat

    cases = [(1, [workloads.named("h", (0,)), workloads.named("rz", (0,), [0.3])]),
             (2, [workloads.named("h", (0,)), workloads.named("cx", (0, 1), ncontrols=1)]),
             (3, [])]
    for n, ops in cases:
        plan = helpers.host_plan(n, ops, precision)
        assert len(plan["passes"]) == (1 if ops else 0)
        got = helpers.interpret(plan, oracle.zero_state(n))
        assert np.abs(got - oracle.simulate(n, ops)).max() < 1e-15
    plan = helpers.host_plan(nat.QFVM_MAX_QUBITS, [workloads.named("h", (nat.QFVM_MAX_QUBITS - 1,))], precision)
    assert len(plan["passes"]) == 1
    for n in (0, nat.QFVM_MAX_QUBITS + 1):
        with pytest.raises(nat.QfvmError) as err:
            helpers.host_plan(n, [workloads.named("h", (0,))], precision)
        assert "qubit count out of range" in str(err.value)
