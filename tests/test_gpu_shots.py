"""Per-shot trajectories on the GPU (qfvm_simulate_shots, the drop-in's
route for circuits with operations after a measurement): the reference's own
mid-circuit cases (golden counts and last-shot states), then random circuits
with mid-circuit measurement of 1-3 qubits, resets and classically
controlled blocks against the oracle, outcome by outcome for the same
uniforms; small (whole-state) and tiled states."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import ir, qfvm, workloads

pytestmark = pytest.mark.gpu

named = workloads.named


def draws(ops):
    return ir.program_draws(ops)


def test_reference_mid_circuit_cases(golden):
    meta, states = golden
    for case in meta["mid_circuit"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        psi = np.zeros(0, dtype=np.complex128)
        out, final = qfvm._shots(case["n"], case["cbits"], ops, psi, case["shots"])
        counts = {}
        for v in out.tolist():
            counts[str(v)] = counts.get(str(v), 0) + 1
        assert counts == case["counts"], case["tag"]
        assert np.max(np.abs(final - states["mid_" + case["tag"]])) < 1e-13, case["tag"]


def random_program(n, ncb, seed, depth=4):
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(depth):
        ops += workloads.random_layers(n, 1, seed=seed * 100 + layer)
        k = int(rng.integers(1, 4))
        qs = [int(q) for q in rng.choice(n, size=k, replace=False)]
        cs = [int(c) for c in rng.choice(ncb, size=k, replace=False)]
        ops.append(ir.Op("measure", ir.OP_MEASURE, qbits=qs, cbits=cs))
        if layer % 2 == 1:
            rq = [int(q) for q in rng.choice(n, size=int(rng.integers(1, 3)), replace=False)]
            ops.append(ir.Op("reset", ir.OP_RESET, qbits=rq))
        cb = [int(c) for c in rng.choice(ncb, size=2, replace=False)]
        body = [named("x", (int(rng.integers(n)),)), named("h", (int(rng.integers(n)),)),
                ir.Op("rz", ir.OP_RZ, (int(rng.integers(n)),), 0, (float(rng.uniform(0, 6)),))]
        ops.append(ir.Op("cif", ir.OP_CIF, cbits=cb, condition=int(rng.integers(4)), body=body))
    ops.append(ir.Op("measure", ir.OP_MEASURE, qbits=list(range(min(n, 4))), cbits=list(range(min(n, 4)))))
    return ops


@pytest.mark.parametrize("n", [5, 13])
def test_random_trajectories_match_oracle(n):
    ncb = 6
    ops = random_program(n, ncb, seed=n)
    shots = 24
    qfvm.set_seed(11)
    out, final = qfvm._shots(n, ncb, ops, np.zeros(0, dtype=np.complex128), shots)
    uni = qfvm.last_uniforms.reshape(shots, draws(ops))
    ref_out, ref_final = oracle.simulate_shots(n, ops, ncb, uni)
    assert out.tolist() == ref_out
    assert np.max(np.abs(final - ref_final)) < 1e-12
    assert abs(np.vdot(final, final).real - 1.0) < 1e-12


def test_input_state_and_chunk_of_one():
    n, ncb = 6, 4
    ops = random_program(n, ncb, seed=3, depth=2)
    psi = helpers.random_state(n, 4)
    qfvm.set_seed(5)
    out, final = qfvm._shots(n, ncb, ops, psi.copy(), 3)
    uni = qfvm.last_uniforms.reshape(3, draws(ops))
    ref_out, ref_final = oracle.simulate_shots(n, ops, ncb, uni, psi_in=psi)
    assert out.tolist() == ref_out
    assert np.max(np.abs(final - ref_final)) < 1e-12
