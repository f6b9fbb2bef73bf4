"""The drop-in ``qfvm`` module (same names and semantics as pyquafu's pybind
module) on the GPU engine."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import qfvm, workloads

pytestmark = pytest.mark.gpu


def proto(n, ops, measures=None):
    return workloads.as_protocol(n, ops, measures)


def test_counts_match_reference(golden):
    meta, _ = golden
    for case in meta["counts"]:
        ops = [helpers.op_from_json(d) for d in case["ops"] if d["kind"] < 40]
        measures = [tuple(m) for m in case["measures"]]
        counts, psi = qfvm.simulate_circuit(proto(case["n"], ops, measures), np.zeros(0, complex), case["shots"])
        assert {str(k): v for k, v in counts.items()} == case["counts"], case["tag"]


def test_sampling_statevec_reference(golden):
    meta, _ = golden
    for case in meta["sampling"]:
        psi = np.zeros(1 << case["n"], dtype=np.complex128)
        psi[case["index"]] = 1.0
        meas = {q: c for q, c in case["measures"]}
        assert qfvm.sampling_statevec(meas, psi, case["shots"]) == case["counts"]


def test_seeded_counts_replay_on_oracle():
    n = 12
    ops = workloads.random_layers(n, 20, seed=0)
    measures = [(q, q) for q in range(n)]
    qfvm.set_seed(0)
    counts, psi = qfvm.simulate_circuit(proto(n, ops, measures), None, 4096)
    u = qfvm.last_uniforms.copy()
    ref_psi = oracle.simulate(n, ops)
    assert np.abs(psi - ref_psi).max() <= 1e-12
    ref_counts = {}
    for b in oracle.bitstrings(oracle.sample_indices(ref_psi, u), measures):
        ref_counts[int(b, 2)] = ref_counts.get(int(b, 2), 0) + 1
    assert counts == ref_counts


def test_inplace_semantics():
    n = 6
    psi = helpers.random_state(n, 1)
    keep = psi
    op = workloads.named("h", (2,))
    out = qfvm.applyop_statevec(workloads._ProtoGate(op), psi)
    assert out is keep
    ref = oracle.simulate(n, [op], helpers.random_state(n, 1))
    assert np.abs(out - ref).max() <= 1e-12
    counts, out2 = qfvm.simulate_circuit(proto(n, [op]), psi, 0)
    assert out2 is keep and counts == {}


def test_expect_statevec(golden):
    from types import SimpleNamespace

    meta, states = golden
    case = [c for c in meta["cases"] if c["tag"] == "allgates_n9"][0]
    paulis = [SimpleNamespace(paulistr=p, pos=pos) for p, pos in case["paulis"]]
    got = qfvm.expect_statevec(states["allgates_n9__out"], paulis)
    np.testing.assert_allclose(got, case["expect"], atol=1e-12, rtol=0)


def test_gpu_entry_returns_state():
    n = 8
    ops = workloads.random_layers(n, 4, seed=4)
    psi = qfvm.simulate_circuit_gpu(proto(n, ops))
    assert np.abs(psi - oracle.simulate(n, ops)).max() <= 1e-12


def test_errors_are_raised_not_crashes():
    with pytest.raises(Exception):
        qfvm.simulate_circuit(proto(3, [workloads.named("h", (3,))]), None, 0)

    class M:
        name = "measure"
        qbits = [0]
        cbits = [0]

    # a gate after a measurement takes the per-shot branch: it needs shots
    pc = proto(2, [workloads.named("h", (0,))])
    pc.instructions = [M()] + pc.instructions
    with pytest.raises(qfvm.QfvmError):
        qfvm.simulate_circuit(pc, None, 0)
    counts, psi = qfvm.simulate_circuit(pc, None, 10)
    assert counts == {0: 10} and abs(abs(psi[0]) - 2 ** -0.5) < 1e-15

    class R:
        name = "reset"
        pos = [5]

    pc.instructions = [R()] + pc.instructions
    with pytest.raises(qfvm.QfvmError):
        qfvm.simulate_circuit(pc, None, 10)


class _Pauli:
    def __init__(self, paulistr, pos):
        self.paulistr, self.pos = paulistr, pos


def test_reference_frontend_calls_replayed(golden):
    """The calls quafu's own front end (quafu.simulate -> SVSimulator.run,
    quafu/simulators/simulator.py:90-145) made into the reference qfvm module
    when tests/golden/make_golden.py ran it, replayed on this module with the
    same arguments: same counts, same statevector (in place when an input
    state is given), same expectation values."""
    meta, states = golden
    calls = meta["frontend"]
    assert [c["fn"] for c in calls].count("simulate_circuit") == 3
    for c in calls:
        if c["fn"] == "simulate_circuit":
            ci = c["circuit"]
            ops = [helpers.op_from_json(d) for d in ci["ops"] if d["kind"] < 40]
            circ = workloads.ProtoCircuit(ci["n"], ops, [tuple(m) for m in ci["measures"]] or None, ci["cbits_num"])
            psi_in = states[c["input"]].copy() if c["input"] else np.array([], dtype=np.complex128)
            counts, psi = qfvm.simulate_circuit(circ, psi_in, c["shots"])
            if c["input"]:
                assert psi is psi_in
            assert {str(k): v for k, v in counts.items()} == c["counts"]
            assert np.abs(psi - states[c["output"]]).max() <= 1e-12
        else:
            paulis = [_Pauli(p, pos) for p, pos in c["paulis"]]
            got = qfvm.expect_statevec(states[c["input"]].copy(), paulis)
            np.testing.assert_allclose(got, c["result"], atol=1e-12, rtol=0)
