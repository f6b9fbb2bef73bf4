"""The CPU oracle (oracle/qsv_oracle.c) against golden outputs of the
reference's own qfvm module (tests/golden/make_golden.py)."""

import numpy as np
import pytest

import helpers
import oracle


def test_circuits_match_reference(golden):
    meta, states = golden
    for case in meta["cases"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        psi_in = states.get(f"{case['tag']}__in")
        got = oracle.simulate(case["n"], [o for o in ops if o.is_gate], psi_in)
        ref = states[f"{case['tag']}__out"]
        err = np.abs(got - ref).max()
        assert err < 1e-13, (case["tag"], err)


def test_expectations_match_reference(golden):
    meta, states = golden
    from types import SimpleNamespace

    for case in meta["cases"]:
        if "paulis" not in case:
            continue
        psi = states[f"{case['tag']}__out"]
        paulis = [SimpleNamespace(paulistr=p, pos=pos) for p, pos in case["paulis"]]
        got = oracle.expect_statevec(psi, paulis)
        np.testing.assert_allclose(got, case["expect"], atol=1e-13, rtol=0)


def test_single_gates_match_reference(golden):
    meta, states = golden
    for i, case in enumerate(meta["apply"]):
        op = helpers.op_from_json(case["op"])
        psi = states[f"apply_{i}__in"].copy()
        oracle.apply_op(psi, op)
        err = np.abs(psi - states[f"apply_{i}__out"]).max()
        assert err < 1e-14, (case["tag"], err)


def _assemble(assembly, gate_grads):
    return [sum(c * gate_grads[i] for i, c in row) for row in assembly]


def test_gradients_match_reference(golden):
    meta, _ = golden
    for case in meta["gradients"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        slots = [o.slot for o in ops]
        terms = [(c, p, pos) for c, p, pos in case["terms"]]
        nslot = max(slots) + 1
        adj = oracle.grad_adjoint(case["n"], ops, slots, terms)
        ps = oracle.grad_param_shift(case["n"], ops, slots, terms)
        e = oracle.energy(case["n"], ops, terms)
        assert abs(e - case["energy"]) < 1e-12
        gate_adj = np.zeros(nslot)
        gate_adj[: len(adj)] = adj
        np.testing.assert_allclose(_assemble(case["assembly"], gate_adj), case["adjoint"], atol=1e-11)
        gate_ps = np.zeros(nslot)
        gate_ps[: len(ps)] = ps
        np.testing.assert_allclose(_assemble(case["assembly"], gate_ps), case["param_shift"], atol=1e-11)


def test_sampling_format_basis_states(golden):
    meta, _ = golden
    for case in meta["sampling"]:
        psi = np.zeros(1 << case["n"], dtype=np.complex128)
        psi[case["index"]] = 1.0
        meas = [tuple(m) for m in case["measures"]]
        u = np.linspace(0.01, 0.99, case["shots"])
        assert oracle.measure_counts(psi, meas, u) == case["counts"]


def test_sampling_scan_semantics():
    rng = np.random.default_rng(3)
    psi = rng.normal(size=64) + 1j * rng.normal(size=64)
    psi /= np.linalg.norm(psi)
    cdf = oracle.sequential_cdf(psi)
    u = np.concatenate([rng.random(200), cdf[:10], [0.0, np.nextafter(cdf[-1], 2.0), 1.0]])
    idx = oracle.sample_indices(psi, u)
    expect = [int(np.searchsorted(cdf, r, side="right")) for r in u]  # first k with r < cdf[k]
    assert [int(i) for i in idx] == expect
    assert int(idx[-1]) == psi.size  # r >= total -> index 2^n (loop end)
    # the single-walk variant (shots by ascending uniform) gives the same indices
    assert np.array_equal(oracle.sample_indices_sorted(psi, u), idx)
    big = rng.normal(size=1 << 12) + 1j * rng.normal(size=1 << 12)
    big /= np.linalg.norm(big)
    ub = np.concatenate([rng.random(3000), oracle.sequential_cdf(big)[::97], [1.0, 0.0, 0.5, 0.5]])
    assert np.array_equal(oracle.sample_indices_sorted(big, ub), oracle.sample_indices(big, ub))


def test_known_answers_bell():
    # tests/quafu/simulator/basis_test.py: Bell state probabilities
    from pyquafu_gb300 import workloads

    psi = oracle.simulate(2, [workloads.named("h", (0,)), workloads.named("cx", (0, 1), ncontrols=1)])
    np.testing.assert_allclose(np.abs(psi) ** 2, [0.5, 0, 0, 0.5], atol=1e-15)


def test_mid_circuit_golden(golden):
    """Per-shot trajectories (qfvm.cpp:104-133) restated by the oracle agree
    with the reference's counts and last-shot states; the circuits are the
    reference's own classic_test.py cases (deterministic outcomes)."""
    meta, states = golden
    rng = np.random.default_rng(0)
    for case in meta["mid_circuit"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        nd = sum(1 for o in ops if o.kind in (40, 41))
        if case["final_measure"]:
            continue
        outcomes, psi = oracle.simulate_shots(case["n"], ops, case["cbits"], rng.random((case["shots"], nd)))
        counts = {}
        for v in outcomes:
            counts[str(v)] = counts.get(str(v), 0) + 1
        assert counts == case["counts"], case["tag"]
        assert np.max(np.abs(psi - states["mid_" + case["tag"]])) < 1e-13, case["tag"]


def test_outcome_choice_rule():
    # first outcome m with u * total < cum[m]; zero-probability outcomes are
    # never chosen, even at u = 0 or just below 1
    assert oracle.choose_outcome([0.0, 0.5, 0.5], 0.0) == 1
    assert oracle.choose_outcome([0.25, 0.25, 0.5, 0.0], 0.5) == 2
    assert oracle.choose_outcome([0.25, 0.25, 0.5, 0.0], 0.9999999999999999) == 2
    assert oracle.choose_outcome([1.0, 0.0], 0.3) == 0


def test_noise_golden(golden):
    """Noisy trajectories (NoiseSVSimulator) restated by the oracle replay the
    reference's seeded channel draws: averaged Pauli expectations and, where
    the final state is a basis state, the counts."""
    meta, _ = golden
    for case in meta["noise"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        uni = helpers.noise_uniforms(ops, case["shots"], case["seed"])
        terms = helpers.noise_terms(case["terms"])
        samples, expv = oracle.simulate_noise(case["n"], ops, uni, terms=terms)
        np.testing.assert_allclose(expv.mean(axis=0), case["pauli_expects"], atol=1e-12, err_msg=case["tag"])
        if "counts" in case:
            strings = oracle.bitstrings(samples, [tuple(m) for m in case["measures"]])
            counts = {}
            for st in strings:
                counts[st] = counts.get(st, 0) + 1
            assert counts == case["counts"], case["tag"]


def test_frontend_calls_match_oracle(golden):
    """The recorded calls of quafu's front end into qfvm, replayed on the
    oracle: the recorded circuits (as read by pyquafu_gb300.ir) give the
    recorded states, and the recorded Pauli terms the recorded values."""
    meta, states = golden
    for c in meta["frontend"]:
        if c["fn"] == "simulate_circuit":
            ops = [helpers.op_from_json(d) for d in c["circuit"]["ops"] if d["kind"] < 40]
            psi_in = states[c["input"]] if c["input"] else None
            got = oracle.simulate(c["circuit"]["n"], ops, psi_in)
            assert np.abs(got - states[c["output"]]).max() < 1e-13
        else:
            psi = states[c["input"]]
            got = [oracle.expect_pauli(psi, p, pos) for p, pos in c["paulis"]]
            np.testing.assert_allclose(got, c["result"], atol=1e-13, rtol=0)
