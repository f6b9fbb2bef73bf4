"""The autotuner on the GPU: every compiled shape it times gives the same
numbers (complex128 parity with the oracle under the chosen shape; batched
complex64 results within 1e-5 of complex128)."""

import numpy as np
import pytest

import oracle
from pyquafu_gb300 import autotune, workloads
from pyquafu_gb300.batch import BatchSession
from pyquafu_gb300.engine import DeviceState, Plan

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def private_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("QFVM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    yield
    for prec in ("c128", "c64", "c128_ds"):
        for kind in autotune.KINDS:
            for n in range(0, 35):
                autotune.set_shape(prec, kind, n, None)


@pytest.mark.parametrize("precision", ["c128", "c64", "c128_ds"])
def test_every_plan_shape_matches_oracle(precision):
    n = 16
    ops = workloads.random_layers(n, 8, seed=2, extras=True)
    ref = oracle.simulate(n, ops)
    tol = 1e-12 if precision != "c64" else 2e-5
    st = DeviceState(n, precision)
    for shape in autotune.candidates(precision, 0):
        plan = Plan(n, ops, precision, *shape)
        st.set_zero()
        plan.run(st)
        assert np.max(np.abs(st.download() - ref)) < tol, shape
        plan.close()
    st.close()
    r = autotune.tune_plan(n, ops, precision)
    assert tuple(r["shape"]) in autotune.candidates(precision, 0)
    assert autotune.current(precision, 0, n) == tuple(r["shape"])


def test_tune_batch_group_and_rerun():
    n, items = 13, 8
    enc = np.random.default_rng(0).uniform(-np.pi, np.pi, n)
    ops, _ = workloads.hea(n, 3, seed=0, encode=enc)
    slots = max(o.slot for o in ops) + 1
    v = np.random.default_rng(1).uniform(-np.pi, np.pi, (items, slots))
    obs = [(1.0, "Z", [0])]
    r = autotune.tune_batch_group(n, ops, v, obs, "c64", reps=1)
    assert tuple(r["forward"]) in autotune.candidates("c64", 0)
    assert tuple(r["reverse"]) in autotune.candidates("c64", 1)
    out = {}
    for prec in ("c64", "c128"):
        with BatchSession(prec, grads=True) as bs:
            bs.add_group(n, ops, obs, items, slots)
            out[prec] = bs.run([v], grads=True)
    np.testing.assert_allclose(out["c64"][0][0], out["c128"][0][0], atol=1e-5)
    np.testing.assert_allclose(out["c64"][1][0], out["c128"][1][0], atol=1e-5)


def test_every_adjoint_shape_matches():
    from pyquafu_gb300 import gradients

    n = 14
    ops, _ = workloads.hea(n, 3, seed=4)
    terms = workloads.zz_x_hamiltonian(n, seed=4)
    e0, g0 = gradients.adjoint(n, ops, terms, "c128")
    for prec, tol in (("c128", 1e-10), ("c128_ds", 1e-10), ("c64", 1e-5)):
        for shape in autotune.candidates(prec, 1):
            autotune.set_shape(prec, 1, n, shape)
            e, g = gradients.adjoint(n, ops, terms, prec)
            assert abs(e - e0) < tol and np.max(np.abs(g - g0)) < tol, (prec, shape)
