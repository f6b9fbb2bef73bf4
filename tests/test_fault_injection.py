"""Failure paths exercised by injection (qfvm_test_fault): an allocation
that fails, a kernel stage that reports an error before its launch, and a
tile-copy wait of the specialised passes that runs out.  Nothing faults the
GPU: the first two make the host wrapper return the error without calling
CUDA; the third makes each pass expect 16 bytes that no copy brings, so its
bounded wait gives up after a short limit and the kernel returns with
QFVM_ERR_TIMEOUT in its status word.  The engine must report the status
with its message, leave no half-made object behind, and keep working
afterwards (checked against the oracle)."""

import numpy as np
import pytest

import oracle
from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import engine, workloads

FAULT_NONE, FAULT_ALLOC, FAULT_STAGE, FAULT_WAIT = 0, 1, 2, 3


@pytest.fixture(autouse=True)
def disarm():
    yield
    nat.load().qfvm_test_fault(FAULT_NONE, 0)


def test_fault_hook_argument_checks():
    lib = nat.load()
    assert lib.qfvm_test_fault(7, 1) == nat.QFVM_ERR_INVALID
    assert b"fault kind" in lib.qfvm_last_error()
    assert lib.qfvm_test_fault(FAULT_ALLOC, 0) == nat.QFVM_ERR_INVALID
    assert lib.qfvm_test_fault(FAULT_WAIT, 20000) == nat.QFVM_ERR_INVALID  # limits above 10 s refused
    assert lib.qfvm_test_fault(FAULT_NONE, 0) == 0


@pytest.mark.gpu
def test_injected_allocation_failure_then_recovery():
    from pyquafu_gb300.builder import build

    build()
    lib = nat.load()
    n = 14
    ops = workloads.random_layers(n, 4, seed=21, extras=True)
    assert lib.qfvm_test_fault(FAULT_ALLOC, 1) == 0
    with pytest.raises(nat.QfvmError) as err:
        engine.DeviceState(n, "c128")
    assert err.value.status == nat.QFVM_ERR_NOMEM
    assert "state allocation" in str(err.value)
    # the hook disarmed itself: the same request now succeeds and computes
    st = engine.DeviceState(n, "c128").set_zero()
    st.apply(ops)
    assert np.abs(st.download() - oracle.simulate(n, ops)).max() <= 1e-12
    # a failing plan allocation (its device records)
    assert lib.qfvm_test_fault(FAULT_ALLOC, 1) == 0
    with pytest.raises(nat.QfvmError) as err:
        engine.Plan(n, ops, "c128")
    assert err.value.status == nat.QFVM_ERR_NOMEM
    plan = engine.Plan(n, ops, "c128")
    st.set_zero()
    plan.run(st)
    assert np.abs(st.download() - oracle.simulate(n, ops)).max() <= 1e-12
    plan.close()
    st.close()


@pytest.mark.gpu
def test_injected_stage_failure_then_recovery():
    lib = nat.load()
    n = 16
    ops = workloads.random_layers(n, 6, seed=22, extras=True)
    plan = engine.Plan(n, ops, "c128")
    assert plan.stats()["passes"] >= 2
    st = engine.DeviceState(n, "c128").set_zero()
    assert lib.qfvm_test_fault(FAULT_STAGE, 2) == 0  # the second pass of the next run
    with pytest.raises(nat.QfvmError) as err:
        plan.run(st)
    assert err.value.status == nat.QFVM_ERR_CUDA
    assert "injected kernel-stage failure" in str(err.value)
    # the context is intact: a fresh run gives the oracle's state
    st.set_zero()
    plan.run(st)
    assert np.abs(st.download() - oracle.simulate(n, ops)).max() <= 1e-12
    plan.close()
    st.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["c128", "c128_ds", "c64"])
def test_tile_copy_wait_runs_out_then_recovery(precision):
    lib = nat.load()
    n = 15
    ops = workloads.random_layers(n, 4, seed=23, extras=True)
    plan = engine.Plan(n, ops, precision)
    st = engine.DeviceState(n, precision).set_zero()
    plan.run(st)
    st.download()  # compiles the specialised passes
    assert plan.jit_passes() > 0
    assert lib.qfvm_test_fault(FAULT_WAIT, 50) == 0  # 50 ms limit per wait
    st.set_zero()
    plan.run(st)
    with pytest.raises(nat.QfvmError) as err:
        st.download()
    assert err.value.status == nat.QFVM_ERR_TIMEOUT
    assert "gave up waiting" in str(err.value)
    assert lib.qfvm_test_fault(FAULT_NONE, 0) == 0
    # the context is intact: a fresh run gives the oracle's state
    st.set_zero()
    plan.run(st)
    tol = 1e-5 if precision == "c64" else 1e-12
    assert np.abs(st.download() - oracle.simulate(n, ops)).max() <= tol
    plan.close()
    st.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["c128", "c128_ds", "c64"])
def test_bounds_checked_passes_run_clean(monkeypatch, precision):
    """QFVM_BOUNDS_CHECK=1 (index-guard build of the specialised passes):
    every access is checked against its buffer; a correct plan reports no
    QFVM_ERR_BOUNDS and computes the oracle's state, one-state passes with a
    shared-memory step and an adjoint reverse sweep alike."""
    from pyquafu_gb300 import gradients

    monkeypatch.setenv("QFVM_BOUNDS_CHECK", "1")
    n = 15
    rng = np.random.default_rng(5)
    u, _ = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
    ops = workloads.random_layers(n, 4, seed=24, extras=True)
    ops.append(workloads.matrix_gate("u2", (2, 11), u))
    plan = engine.Plan(n, ops, precision)
    st = engine.DeviceState(n, precision).set_zero()
    plan.run(st)
    got = st.download()
    assert plan.jit_passes() > 0
    tol = 1e-5 if precision == "c64" else 1e-12
    assert np.abs(got - oracle.simulate(n, ops)).max() <= tol
    plan.close()
    st.close()
    aops, _ = workloads.hea(n, 3, seed=2)
    terms = workloads.zz_x_hamiltonian(n, seed=2)
    _, g = gradients.adjoint(n, aops, terms, precision)
    ref = oracle.grad_adjoint(n, aops, [o.slot for o in aops], terms)
    assert np.abs(g - ref).max() <= (1e-4 if precision == "c64" else 1e-10)
