"""Noisy trajectories on the GPU (qfvm_simulate_noise, the NoiseSVSimulator
drop-in): the reference's seeded runs (golden averaged expectations and
counts), random circuits with unitary and Kraus channels against the oracle
shot by shot (Kraus sets whose Gram matrices are diagonal and ones that are
not), and the drop-in class on protocol objects."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import ir, noise, workloads

pytestmark = pytest.mark.gpu

X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]])
Z = np.diag([1.0, -1.0]).astype(complex)
I2 = np.eye(2, dtype=complex)


def amp_damp(p):
    return [np.array([[1, 0], [0, np.sqrt(1 - p)]], dtype=complex), np.array([[0, np.sqrt(p)], [0, 0]], dtype=complex)]


def test_reference_noise_cases(golden):
    meta, _ = golden
    for case in meta["noise"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        uni = helpers.noise_uniforms(ops, case["shots"], case["seed"])
        terms = helpers.noise_terms(case["terms"])
        samples, expv = noise.simulate_noise(case["n"], ops, case["shots"], terms=terms, uniforms=uni)
        np.testing.assert_allclose(expv.mean(axis=0), case["pauli_expects"], atol=1e-12, err_msg=case["tag"])
        if "counts" in case:
            counts = {}
            for st in oracle.bitstrings(samples, [tuple(m) for m in case["measures"]]):
                counts[st] = counts.get(st, 0) + 1
            assert counts == case["counts"], case["tag"]


def random_noisy(n, seed):
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(4):
        ops += workloads.random_layers(n, 1, seed=seed * 10 + layer)
        for _ in range(2):
            q = int(rng.integers(n))
            p = float(rng.uniform(0.05, 0.5))
            ops.append(ir.channel_op(ir.OP_UCHANNEL, q, [X, Y, Z, I2], [p / 3, p / 3, p / 3, 1 - p]))
            ops.append(ir.channel_op(ir.OP_KRAUS, int(rng.integers(n)), amp_damp(float(rng.uniform(0.1, 0.6)))))
    return ops


@pytest.mark.parametrize("n", [5, 13])
def test_random_noisy_circuits_match_oracle(n):
    ops = random_noisy(n, seed=n)
    shots = 12
    uni = np.random.default_rng(n).random((shots, ir.noise_draws(ops)))
    terms = [(1.0, "Z", [0]), (0.5, "XY", [1, 2]), (-0.7, "ZZ", [0, n - 1])]
    samples, expv = noise.simulate_noise(n, ops, shots, terms=terms, uniforms=uni)
    ref_s, ref_e = oracle.simulate_noise(n, ops, uni, terms=terms)
    assert samples.tolist() == ref_s
    np.testing.assert_allclose(expv, ref_e, atol=1e-12)


def rotated_kraus(theta, seed):
    """Amplitude damping followed by a random unitary V: K_i V.  Its Gram
    matrices V^dagger K_i^dagger K_i V have off-diagonal entries, so the
    kernels' norm sums need the cross term sum conj(a) c."""
    rng = np.random.default_rng(seed)
    z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    v, _ = np.linalg.qr(z)
    return [k @ v for k in amp_damp(theta)]


@pytest.mark.parametrize("n", [6, 15])
def test_kraus_channels_with_cross_terms(n):
    rng = np.random.default_rng(40 + n)
    ops = []
    for layer in range(3):
        ops += workloads.random_layers(n, 1, seed=500 + layer)
        for _ in range(3):
            ops.append(ir.channel_op(ir.OP_KRAUS, int(rng.integers(n)),
                                     rotated_kraus(float(rng.uniform(0.1, 0.7)), int(rng.integers(1 << 30)))))
    shots = 16
    uni = np.random.default_rng(n).random((shots, ir.noise_draws(ops)))
    terms = [(1.0, "Z", [0]), (0.5, "XX", [1, 2])]
    samples, expv = noise.simulate_noise(n, ops, shots, terms=terms, uniforms=uni)
    ref_s, ref_e = oracle.simulate_noise(n, ops, uni, terms=terms)
    assert samples.tolist() == ref_s
    np.testing.assert_allclose(expv, ref_e, atol=1e-12)


class _Gate:
    def __init__(self, q, m):
        self.name = "G"
        self.pos = [q]
        self.paras = []
        self._paras = []
        self.matrix = m


class UnitaryChannel:
    def __init__(self, q, mats, probs):
        self.pos = [q]
        self.gatelist = [_Gate(q, m) for m in mats]
        self.probs = probs


class KrausChannel:
    def __init__(self, q, mats):
        self.pos = [q]
        self.gatelist = [_Gate(q, m) for m in mats]


def test_dropin_simulator_on_protocol_objects():
    n = 3
    circ = workloads.ProtoCircuit(n, [workloads.named("h", (0,)), workloads.named("cx", (0, 1), ncontrols=1)])
    circ.instructions += [UnitaryChannel(1, [X, I2], [0.3, 0.7]), KrausChannel(2, amp_damp(0.4))]
    circ.measures = {0: 0, 1: 1, 2: 2}

    class P:
        def __init__(self, s, pos, c):
            self.paulistr, self.pos, self.coeff = s, pos, c

    class H:
        paulis = [P("Z", [1], 1.0), P("XX", [0, 1], 0.5)]

    shots = 50
    ops = [ir.read_noisy_op(i) for i in circ.instructions]
    uni = np.random.default_rng(3).random((shots, ir.noise_draws(ops)))
    res = noise.NoiseSVSimulator().run(circ, shots=shots, hamiltonian=H(), uniforms=uni)
    res = res if isinstance(res, dict) else res.__dict__
    ref_s, ref_e = oracle.simulate_noise(n, ops, uni, terms=[(1.0, "Z", [1]), (0.5, "XX", [0, 1])])
    counts = {}
    for st in oracle.bitstrings(ref_s, [(0, 0), (1, 1), (2, 2)]):
        counts[st] = counts.get(st, 0) + 1
    assert res["counts"] == counts
    np.testing.assert_allclose(res["pauli_expects"], ref_e.mean(axis=0), atol=1e-12)
