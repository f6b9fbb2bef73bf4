"""GPU engine parity against the reference's golden outputs and the CPU
oracle.  Tolerances: complex128 per-amplitude |delta| <= 1e-12;
complex64 per-amplitude |delta| <= 1e-5; sampled indices bit-exact."""

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import engine, workloads

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from pyquafu_gb300.builder import build

    build()


def run(n, ops, precision="c128", psi_in=None, T=0, R=0):
    st = engine.DeviceState(n, precision)
    if psi_in is None:
        st.set_zero()
    else:
        st.upload(psi_in)
    if T or R:
        plan = engine.Plan(n, ops, precision, T, R)
        plan.run(st)
    else:
        st.apply(ops)
    out = st.download()
    st.close()
    return out


def test_golden_circuits(golden):
    meta, states = golden
    for case in meta["cases"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        got = run(case["n"], [o for o in ops if o.is_gate], psi_in=states.get(f"{case['tag']}__in"))
        err = np.abs(got - states[f"{case['tag']}__out"]).max()
        assert err <= TOL128, (case["tag"], err)


def test_golden_single_gates(golden):
    meta, states = golden
    for i, case in enumerate(meta["apply"]):
        op = helpers.op_from_json(case["op"])
        got = run(5, [op], psi_in=states[f"apply_{i}__in"])
        err = np.abs(got - states[f"apply_{i}__out"]).max()
        assert err <= TOL128, (case["tag"], err)


@pytest.mark.parametrize("T,R", [(11, 4), (12, 4), (12, 5), (12, 3), (11, 3)])
def test_tile_shapes_c128(T, R):
    for n in (T, T + 3):
        ops = workloads.random_layers(n, 6, seed=1000 + n, extras=True, extra_rate=0.6)
        got = run(n, ops, "c128", T=T, R=R)
        err = np.abs(got - oracle.simulate(n, ops)).max()
        assert err <= TOL128, (n, T, R, err)


@pytest.mark.parametrize("T,R", [(11, 4), (12, 4), (12, 5), (12, 3)])
def test_tile_shapes_double_single(T, R):
    # complex128 storage with double-single arithmetic: same 1e-12 bound
    for n in (T, T + 3):
        ops = workloads.random_layers(n, 6, seed=3000 + n, extras=True, extra_rate=0.6)
        got = run(n, ops, "c128_ds", T=T, R=R)
        err = np.abs(got - oracle.simulate(n, ops)).max()
        assert err <= TOL128, (n, T, R, err)


def test_golden_circuits_double_single(golden):
    meta, states = golden
    for case in meta["cases"]:
        ops = [helpers.op_from_json(d) for d in case["ops"]]
        got = run(case["n"], [o for o in ops if o.is_gate], "c128_ds", psi_in=states.get(f"{case['tag']}__in"))
        err = np.abs(got - states[f"{case['tag']}__out"]).max()
        assert err <= TOL128, (case["tag"], err)


def test_swap_register_order():
    # swaps whose targets land in either register order inside one round
    n = 14
    ops = []
    for a, b in [(0, 3), (3, 0), (12, 5), (5, 12), (13, 1), (2, 11)]:
        ops += [workloads.named("h", (a,)), workloads.named("ry", (b,), (0.4,)),
                workloads.matrix_gate("swap", (a, b), workloads.SWAP)]
    for prec in ("c128", "c128_ds"):
        got = run(n, ops, prec, T=12, R=4)
        assert np.abs(got - oracle.simulate(n, ops)).max() <= TOL128, prec


@pytest.mark.parametrize("T,R", [(12, 5), (13, 5), (12, 4), (13, 4)])
def test_tile_shapes_c64(T, R):
    n = T + 2
    ops = workloads.random_layers(n, 5, seed=2000 + n, extras=True, extra_rate=0.6)
    got = run(n, ops, "c64", T=T, R=R)
    err = np.abs(got - oracle.simulate(n, ops)).max()
    assert err <= TOL64, (n, T, R, err)


def test_all_gate_kinds_tile_pass(golden):
    meta, states = golden
    case = [c for c in meta["cases"] if c["tag"] == "allgates_n12"][0]
    ops = [helpers.op_from_json(d) for d in case["ops"]]
    got = run(12, ops, "c128", T=11, R=4)
    assert np.abs(got - states["allgates_n12__out"]).max() <= TOL128


def test_dense_multi_target_large_state():
    rng = np.random.default_rng(0)
    m = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    ops = [workloads.named("h", (q,)) for q in range(15)]
    ops.append(workloads.matrix_gate("u3q", (14, 1, 7), m))
    ops.append(workloads.matrix_gate("cu", (3, 9), np.array([[0.6, 0.8j], [0.8j, 0.6]]), ncontrols=1))
    ops += [workloads.named("rx", (q,), (0.3 * q,)) for q in range(15)]
    got = run(15, ops)
    assert np.abs(got - oracle.simulate(15, ops)).max() <= TOL128


def _unitary(k, seed):
    rng = np.random.default_rng(seed)
    d = 1 << k
    return np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]


@pytest.mark.parametrize("precision,tol", [("c128", TOL128), ("c128_ds", TOL128), ("c64", TOL64)])
@pytest.mark.parametrize("n", [10, 16])
def test_dense_gates_on_7_to_12_targets(precision, tol, n):
    """Matrix gates on 7, 8 and 12 targets in any order, some controlled
    (the reference's apply_multi_targe_gate_general takes any count,
    statevector.hpp:945-995), in a small state and a tiled one."""
    rng = np.random.default_rng(n)
    ops = [workloads.named("h", (q,)) for q in range(n)]
    for k, nc in ((7, 0), (8, 1), (7, 2)):
        qs = [int(q) for q in rng.permutation(n)[: k + nc]]
        ops.append(workloads.matrix_gate(f"u{k}", qs, _unitary(k, k + nc), ncontrols=nc))
        ops += [workloads.named("ry", (q,), (0.1 + 0.2 * q,)) for q in range(n)]
    if n >= 12:
        qs = [int(q) for q in rng.permutation(n)[:12]]
        ops.append(workloads.matrix_gate("u12", qs, _unitary(12, 3)))
    got = run(n, ops, precision)
    assert np.abs(got - oracle.simulate(n, ops)).max() <= tol


def test_input_state_and_controls_outside_tile():
    n = 16
    psi = helpers.random_state(n, 5)
    ops = [workloads.named("cx", (15, 2), ncontrols=1), workloads.named("ccx", (14, 13, 0), ncontrols=2),
           workloads.named("cp", (12, 1, 0.7), ncontrols=1), workloads.named("rzz", (15, 0), (1.1,)),
           workloads.named("cz", (10, 11), ncontrols=1)]
    ops += workloads.random_layers(n, 3, seed=9)
    got = run(n, ops, psi_in=psi)
    assert np.abs(got - oracle.simulate(n, ops, psi)).max() <= TOL128


def test_expectation_golden(golden):
    meta, states = golden
    for case in meta["cases"]:
        if "paulis" not in case:
            continue
        st = engine.DeviceState(case["n"]).upload(states[f"{case['tag']}__out"])
        got = st.expect([(p, pos) for p, pos in case["paulis"]])
        st.close()
        np.testing.assert_allclose(got, case["expect"], atol=TOL128, rtol=0)


def test_expectation_many_terms():
    n = 18
    psi = helpers.random_state(n, 11)
    rng = np.random.default_rng(1)
    terms = []
    for _ in range(40):
        k = int(rng.integers(1, 4))
        qs = [int(q) for q in rng.choice(n, k, replace=False)]
        terms.append(("".join(rng.choice(list("XYZ"), k)), qs))
    terms += [("Z", [0])] * 3 + [("X", [17])]
    st = engine.DeviceState(n).upload(psi)
    got = st.expect(terms)
    ref = [oracle.expect_pauli(psi, p, q) for p, q in terms]
    np.testing.assert_allclose(got, ref, atol=TOL128, rtol=0)
    np.testing.assert_allclose(st.norm2(), 1.0, atol=TOL128)
    st.close()


def test_expectation_c64():
    n = 16
    psi = helpers.random_state(n, 3)
    st = engine.DeviceState(n, "c64").upload(psi)
    got = st.expect([("ZZ", [0, 1]), ("X", [3]), ("YX", [2, 15])])
    ref = [oracle.expect_pauli(psi, p, q) for p, q in [("ZZ", [0, 1]), ("X", [3]), ("YX", [2, 15])]]
    np.testing.assert_allclose(got, ref, atol=1e-6, rtol=0)
    st.close()


@pytest.mark.parametrize("n", [1, 5, 12, 20])
def test_sampling_bit_exact(n):
    psi = helpers.random_state(n, 100 + n)
    cdf = oracle.sequential_cdf(psi)
    rng = np.random.default_rng(n)
    u = list(rng.random(3000))
    u += [0.0, float(np.nextafter(cdf[-1], 2.0)), float(cdf[-1]), 1.0 - 2.0 ** -53]
    pick = rng.choice(cdf.size, min(cdf.size, 50), replace=False)
    u += [float(cdf[i]) for i in pick]                       # exact CDF values (ties)
    u += [float(np.nextafter(cdf[i], -1.0)) for i in pick]   # one ulp below
    u = np.array(u)
    st = engine.DeviceState(n).upload(psi)
    got = st.sample(u)
    st.close()
    ref = oracle.sample_indices(psi, u)
    assert np.array_equal(got, ref)


def test_sampling_sparse_state():
    n = 14
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[[3, 700, 9000, 16383]] = np.array([0.5, 0.5j, -0.5, 0.5])
    u = np.random.default_rng(0).random(500)
    st = engine.DeviceState(n).upload(psi)
    got = st.sample(u)
    st.close()
    assert np.array_equal(got, oracle.sample_indices(psi, u))


def test_large_state_properties():
    # size-independent checks at a larger size: norm, and U^dagger U = I
    n = 26
    ops = workloads.random_layers(n, 8, seed=3, extras=True)
    st = engine.DeviceState(n).set_zero()
    st.apply(ops)
    assert abs(st.norm2() - 1.0) < 1e-12
    st.apply(helpers.inverse(ops))
    z = st.expect([("Z" * n, list(range(n)))])[0]
    psi0 = st.download()
    st.close()
    assert abs(abs(psi0[0]) - 1.0) < 1e-11
    assert np.abs(psi0[1:]).max() < 1e-11
    assert abs(z - 1.0) < 1e-11
