"""Circuit-specialised tile passes (PTX generated per pass and compiled on
the host) against the interpreting kernels and the oracle, on the same
inputs: one-state passes in complex128 (FP64 and double-single arithmetic)
and complex64 for several tile shapes and both buffering modes; dense, Y,
Hadamard and SWAP gates on the targets of thread-controlled cx (pending
per-thread flips); two-qubit unitaries as shared-memory steps; reverse sweeps with probes (adjoint gradients); batched
groups (per-item coefficients, per-tile probe sums); and per-shot
trajectories whose classically controlled blocks use the active-item mask.
Tolerances: complex128 1e-12 per amplitude, gradients 1e-10; complex64
1e-5."""

import numpy as np
import pytest

import oracle
from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import engine, gradients, ir, qfvm, workloads
from pyquafu_gb300.batch import BatchSession

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c128_ds": 1e-12, "c64": 1e-5}


@pytest.fixture(autouse=True)
def restore_jit():
    yield
    engine.jit_configure(True)


def run_state(n, ops, precision, T, R, jit, nb=1, minb=0):
    engine.jit_configure(jit, nb, minb, 1, 0)
    st = engine.DeviceState(n, precision)
    st.set_zero()
    plan = engine.Plan(n, ops, precision, T, R)
    plan.run(st)
    out = st.download()
    used = plan.jit_passes(1)
    plan.close()
    st.close()
    return out, used


@pytest.mark.parametrize("precision,T,R", [("c128", 11, 3), ("c128", 11, 4), ("c128", 12, 5),
                                           ("c64", 13, 4), ("c64", 12, 5), ("c64", 12, 4),
                                           ("c128_ds", 12, 3), ("c128_ds", 11, 4)])
@pytest.mark.parametrize("nb", [1, 2])
def test_one_state_passes(precision, T, R, nb):
    n = 17
    ops = workloads.random_layers(n, 8, seed=T * 10 + R, extras=True)
    got, used = run_state(n, ops, precision, T, R, True, nb)
    assert used > 0
    interp, used0 = run_state(n, ops, precision, T, R, False)
    assert used0 == 0
    ref = oracle.simulate(n, ops)
    assert np.abs(got - ref).max() < TOL[precision]
    assert np.abs(got - interp).max() < TOL[precision]


def test_thread_controls_and_phases():
    """Controls on thread bits, parities and uniform phases (cz/cp/rzz across
    tile and register bits) in complex128."""
    n = 16
    rng = np.random.default_rng(4)
    ops = []
    for layer in range(6):
        for q in range(n):
            ops.append(workloads.named(["h", "t", "s", "sdg", "x", "y"][int(rng.integers(6))], (q,)))
        for _ in range(n):
            a, b, c = (int(v) for v in rng.choice(n, 3, replace=False))
            kind = ["cx", "cz", "cp", "rzz", "ccx"][int(rng.integers(5))]
            if kind in ("cp", "rzz"):
                ops.append(ir.Op(kind, ir.NAMED_KIND[kind], (a, b), 1 if kind == "cp" else 0,
                                 (float(rng.uniform(0, 6.3)),)))
            elif kind == "ccx":
                ops.append(workloads.named("ccx", (a, b, c), ncontrols=2))
            else:
                ops.append(workloads.named(kind, (a, b), ncontrols=1))
    got, used = run_state(n, ops, "c128", 11, 3, True)
    assert used > 0
    ref = oracle.simulate(n, ops)
    assert np.abs(got - ref).max() < 1e-12


@pytest.mark.parametrize("precision", ["c128", "c64", "c128_ds"])
def test_dense_gates_after_thread_controlled_flips(precision):
    """Random one-qubit unitaries (dense 2x2), Y, Hadamards and SWAPs on the
    targets of cx gates whose controls are thread bits: the pending flips are
    conjugated into dense coefficients, moved by SWAP or materialised."""
    n = 17
    rng = np.random.default_rng(11)
    ops = []
    for layer in range(8):
        for q in range(n):
            z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
            u, _ = np.linalg.qr(z)
            kind = int(rng.integers(4))
            if kind == 0:
                ops.append(workloads.matrix_gate("u", (q,), u))
            elif kind == 1:
                ops.append(workloads.named(["y", "h"][int(rng.integers(2))], (q,)))
            elif kind == 2:
                ops.append(workloads.named(["rx", "ry"][int(rng.integers(2))], (q,), (float(rng.uniform(0, 6.3)),)))
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            ops.append(workloads.named("cx", (int(perm[i]), int(perm[i + 1])), ncontrols=1))
        a, b = (int(v) for v in rng.choice(n, 2, replace=False))
        ops.append(workloads.matrix_gate("swap", (a, b), workloads.SWAP))
    T, R = (12, 4) if precision == "c64" else (11, 4)
    got, used = run_state(n, ops, precision, T, R, True)
    assert used > 0
    ref = oracle.simulate(n, ops)
    assert np.abs(got - ref).max() < TOL[precision]


@pytest.mark.parametrize("precision", ["c128", "c64", "c128_ds"])
def test_shared_memory_steps(precision):
    """Random two-qubit unitaries run as shared-memory steps inside the
    specialised passes (no pass falls back to the interpreting kernel)."""
    from test_jit_host import dense2_circuit

    n = 17
    ops = dense2_circuit(n, 5)
    T, R = (12, 4) if precision == "c64" else (11, 4)
    engine.jit_configure(True)
    st = engine.DeviceState(n, precision)
    st.set_zero()
    plan = engine.Plan(n, ops, precision, T, R)
    plan.run(st)
    got = st.download()
    assert plan.jit_passes(1) == plan.stats()["passes"]
    plan.close()
    st.close()
    assert np.abs(got - oracle.simulate(n, ops)).max() < TOL[precision]


def test_shared_memory_steps_in_reverse_sweeps():
    from test_jit_host import dense2_circuit

    n = 15
    enc = np.random.default_rng(2).uniform(-np.pi, np.pi, n)
    ops, _ = workloads.hea(n, 2, seed=4, encode=enc)
    ops = dense2_circuit(n, 6)[: 3 * n] + ops
    terms = workloads.zz_x_hamiltonian(n, seed=5)
    engine.jit_configure(True)
    e1, g1 = gradients.adjoint(n, ops, terms, "c128")
    engine.jit_configure(False)
    e0, g0 = gradients.adjoint(n, ops, terms, "c128")
    assert abs(e1 - e0) < 1e-12
    np.testing.assert_allclose(g1, g0, atol=1e-10)


@pytest.mark.parametrize("precision", ["c128", "c128_ds", "c64"])
def test_adjoint_reverse_sweep(precision):
    n = 16
    enc = np.random.default_rng(1).uniform(-np.pi, np.pi, n)
    ops, params = workloads.hea(n, 3, seed=2, encode=enc)
    terms = workloads.zz_x_hamiltonian(n, seed=3)
    engine.jit_configure(True)
    e1, g1 = gradients.adjoint(n, ops, terms, precision)
    engine.jit_configure(False)
    e0, g0 = gradients.adjoint(n, ops, terms, precision)
    gtol = 1e-4 if precision == "c64" else 1e-10
    assert abs(e1 - e0) < (1e-5 if precision == "c64" else 1e-12)
    np.testing.assert_allclose(g1, g0, atol=gtol)
    if precision != "c64":
        ref = oracle.grad_adjoint(n, ops, [o.slot for o in ops], terms)
        np.testing.assert_allclose(g1[: len(ref)], ref, atol=1e-10)


def test_batched_groups():
    n = 16
    ops, weights, x, y = workloads.qnn_batch(batch=6, n=n, layers=3, seed=5)
    nslots = max(o.slot for o in ops) + 1
    v = np.random.default_rng(6).uniform(-np.pi, np.pi, (6, nslots))
    out = []
    for jit in (True, False):
        engine.jit_configure(jit)
        with BatchSession("c64", grads=True) as bs:
            bs.add_group(n, ops, [(1.0, "Z", [0])], 6, nslots)
            for _ in range(3):  # direct, captured, replayed
                e, g = bs.run([v], grads=True)
            out.append((e[0], g[0]))
    np.testing.assert_allclose(out[0][0], out[1][0], atol=1e-5)
    np.testing.assert_allclose(out[0][1], out[1][1], atol=1e-4)
    psi = oracle.simulate(n, gradients.bind(ops, v[0]))
    assert abs(out[0][0][0, 0] - oracle.expect_pauli(psi, "Z", [0])) < 1e-5


def test_trajectories_with_classical_control():
    from test_gpu_shots import random_program

    n, ncb, shots = 15, 6, 8
    ops = random_program(n, ncb, seed=21, depth=3)
    res = []
    for jit in (True, False):
        engine.jit_configure(jit)
        qfvm.set_seed(3)
        res.append(qfvm._shots(n, ncb, ops, np.zeros(0, dtype=np.complex128), shots))
    assert res[0][0].tolist() == res[1][0].tolist()
    assert np.abs(res[0][1] - res[1][1]).max() < 1e-12


def test_double_single_passes_chained_as_float_pairs():
    """A double-single plan whose passes are all specialised hands the state
    from pass to pass as float pairs: the first pass converts FP64 to pairs,
    the middle ones move pairs by bulk copies both ways, the last converts
    back.  The final state matches the oracle to 1e-12, and so do runs that
    start from a given state and repeat."""
    import ctypes

    n = 20
    ops = workloads.random_layers(n, 16, seed=31, extras=True)
    plan = engine.Plan(n, ops, "c128_ds")
    assert plan.stats()["passes"] >= 3
    st = engine.DeviceState(n, "c128_ds").set_zero()
    plan.run(st)
    got = st.download()
    assert plan.jit_passes() == plan.stats()["passes"]
    ref = oracle.simulate(n, ops)
    assert np.abs(got - ref).max() <= 1e-12
    # the middle passes neither convert nor store per thread: their PTX reads
    # and writes float pairs through bulk copies only
    lib = nat.load()
    ln = ctypes.c_int64()
    assert lib.qfvm_jit_pass_ptx(plan._h, 1, 1, None, 0, ctypes.byref(ln)) == 0
    buf = ctypes.create_string_buffer(ln.value + 1)
    assert lib.qfvm_jit_pass_ptx(plan._h, 1, 1, buf, ln.value + 1, ctypes.byref(ln)) == 0
    mid = buf.value.decode()
    assert "ld.shared.v2.f64" not in mid and "st.global.cs" not in mid and "cp.async.bulk.global.shared" in mid
    # a second run from the result (state given as FP64 again)
    plan.run(st)
    again = st.download()
    ref2 = oracle.simulate(n, ops, ref)
    assert np.abs(again - ref2).max() <= 1e-12
    plan.close()
    st.close()
