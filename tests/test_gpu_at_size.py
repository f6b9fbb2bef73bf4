"""Parity at the sizes the benchmarks are quoted on, against the oracle run
on the host cores (OpenMP) in the same process.

* 30 qubits, complex128 (16 GiB state): the 40-layer random circuit with
  cz/swap/rzz/ccx extras, seed 0 (1808 gates).  The final state of every
  arithmetic (FP64, double-single, complex64) is compared per amplitude with
  the oracle's, and <Z0 Z1> with the oracle's expect_pauli.
* 20 qubits, complex128: the 20-layer random circuit, seed 0, with 4096
  shots.  Final state per amplitude, sampled indices bit-exact against the
  oracle's sequential scan given the same seeded uniforms, and the counts of
  the drop-in simulate_circuit against the oracle's measure_samples rule.
* 24 qubits, complex128: the 20-layer hardware-efficient ansatz (960
  parameters) with sum a_i Z_i Z_i+1 + sum b_i X_i: the adjoint gradient on
  every parameter against the oracle's adjoint, a subset against central
  finite differences (h = 1e-6) and against the GPU parameter shift.

Tolerances (stated in each assertion): complex128 and double-single
per-amplitude |delta| <= 1e-12; complex64 per-amplitude |delta| <= 1e-6 at
30 qubits (it carries 24-bit arithmetic through 1808 gates); gradients
1e-10 (complex128, double-single) and 1e-4 (complex64).
"""

import numpy as np
import pytest

import oracle
from pyquafu_gb300 import engine, gradients, qfvm, workloads

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64_30Q = 1e-6


@pytest.fixture(scope="module", autouse=True)
def built():
    from pyquafu_gb300.builder import build

    build()
    oracle.build()


def max_abs_diff(a, b, chunk=1 << 24):
    """Largest per-amplitude |a - b| over two equal-length arrays, in chunks
    (keeps the temporaries small at 2^30 amplitudes)."""
    m = 0.0
    for i in range(0, a.size, chunk):
        m = max(m, float(np.abs(a[i:i + chunk] - b[i:i + chunk]).max()))
    return m


@pytest.fixture(scope="module")
def c2_reference():
    n = 30
    ops = workloads.random_layers(n, 40, seed=0, extras=True)
    assert len(ops) == 1808
    psi = oracle.simulate(n, ops)
    zz = oracle.expect_pauli(psi, "ZZ", [0, 1])
    return n, ops, psi, zz


@pytest.mark.parametrize("precision,tol", [("c128", TOL128), ("c128_ds", TOL128), ("c64", TOL64_30Q)])
def test_30q_random_layers_against_oracle(c2_reference, precision, tol):
    n, ops, ref, zz_ref = c2_reference
    st = engine.DeviceState(n, precision).set_zero()
    st.apply(ops)
    zz = float(st.expect([("ZZ", [0, 1])])[0])
    got = st.download()
    st.close()
    err = max_abs_diff(got, ref)
    del got
    print(f"30q {precision}: max per-amplitude |delta| = {err:.3e}, |delta <Z0Z1>| = {abs(zz - zz_ref):.3e}")
    assert err <= tol, (precision, err)
    assert abs(zz - zz_ref) <= tol, (precision, zz, zz_ref)


def test_20q_state_and_4096_shots_bit_exact():
    n, shots = 20, 4096
    ops = workloads.random_layers(n, 20, seed=0)
    assert len(ops) == 20 * (n + n // 2)
    ref = oracle.simulate(n, ops)
    st = engine.DeviceState(n, "c128").set_zero()
    st.apply(ops)
    got = st.download()
    assert np.abs(got - ref).max() <= TOL128
    # sampled indices: the same seeded host uniforms on both sides
    u = np.random.Generator(np.random.MT19937(0)).random(shots)
    idx = st.sample(u)
    st.close()
    assert np.array_equal(idx, oracle.sample_indices(ref, u))
    # the drop-in entry point: counts keyed like qfvm.cpp:93-97
    measures = [(q, q) for q in range(n)]
    circ = workloads.as_protocol(n, ops, measures=measures)
    qfvm.set_seed(0)
    counts, _ = qfvm.simulate_circuit(circ, None, shots)
    ref_counts = oracle.measure_counts(ref, measures, qfvm.last_uniforms)
    assert counts == {int(k, 2): v for k, v in ref_counts.items()}


@pytest.fixture(scope="module")
def c3_reference():
    n, layers = 24, 20
    ops, params = workloads.hea(n, layers, seed=0)
    terms = workloads.zz_x_hamiltonian(n, seed=0)
    assert len(params) == 960 and len(terms) == 47
    ref = oracle.grad_adjoint(n, ops, [o.slot for o in ops], terms)
    return n, ops, params, terms, ref


@pytest.mark.parametrize("precision,tol", [("c128", 1e-10), ("c128_ds", 1e-10), ("c64", 1e-4)])
def test_24q_adjoint_960_parameters_against_oracle(c3_reference, precision, tol):
    n, ops, _, terms, ref = c3_reference
    e, g = gradients.adjoint(n, ops, terms, precision)
    err = float(np.abs(g - ref).max())
    print(f"24q adjoint {precision}: max |delta grad| over {g.size} parameters = {err:.3e}")
    assert g.size == ref.size == 960
    assert err <= tol, (precision, err)


def test_24q_adjoint_finite_differences_and_param_shift(c3_reference):
    n, ops, params, terms, ref = c3_reference
    subset = [0, 1, 23, 24, 480, 481, 958, 959]
    h = 1e-6
    st = engine.DeviceState(n, "c128")
    for k in subset:
        vals = []
        for s in (h, -h):
            p = params.copy()
            p[k] += s
            vals.append(gradients.energy(n, gradients.bind(ops, p), terms, "c128", st))
        fd = (vals[0] - vals[1]) / (2 * h)
        # central differences: O(h^2) truncation plus ~1e-16 / h rounding
        assert abs(fd - ref[k]) <= 1e-7, (k, fd, ref[k])
        shifted = []
        for s in (np.pi / 2, -np.pi / 2):
            p = params.copy()
            p[k] += s
            shifted.append(gradients.energy(n, gradients.bind(ops, p), terms, "c128", st))
        assert abs((shifted[0] - shifted[1]) / 2 - ref[k]) <= 1e-10, k
    st.close()
