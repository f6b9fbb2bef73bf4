"""Batched runs on the GPU (qfvm_batch_*) against the oracle, item by item:
groups of uneven qubit counts in one run, per-item angles bound on the
device, expectation values and adjoint gradients, weighted observables, and
the CUDA-graph replay giving the same numbers as the directly issued run.
Tolerances: complex128 and double-single 1e-10 (values 1e-12), complex64
1e-5."""

import numpy as np
import pytest

import oracle
from pyquafu_gb300 import gradients, workloads
from pyquafu_gb300.batch import BatchSession

pytestmark = pytest.mark.gpu

TOL = {"c128": (1e-12, 1e-10), "c128_ds": (1e-11, 1e-10), "c64": (1e-5, 1e-5)}


def encoded_hea(n, layers, seed):
    enc = np.random.default_rng(seed).uniform(-np.pi, np.pi, n)
    ops, _ = workloads.hea(n, layers, seed=seed, encode=enc)
    return ops, max(o.slot for o in ops) + 1


def oracle_item(n, ops, v, terms):
    bound = gradients.bind(ops, v)
    psi = oracle.simulate(n, bound)
    e = sum(c * oracle.expect_pauli(psi, p, pos) for c, p, pos in terms)
    g = oracle.grad_adjoint(n, bound, [o.slot for o in bound], terms)
    return e, g


@pytest.mark.parametrize("precision", ["c128", "c64", "c128_ds"])
def test_uneven_groups_match_oracle(precision):
    vtol, gtol = TOL[precision]
    ns = [6, 10, 12, 13, 14]
    rng = np.random.default_rng(0)
    terms = [(1.0, "Z", [0])]
    with BatchSession(precision, grads=True) as bs:
        groups = []
        for n in ns:
            ops, ns_ = encoded_hea(n, 2, seed=n)
            items = 3
            bs.add_group(n, ops, terms, items, ns_)
            groups.append((n, ops, rng.uniform(-np.pi, np.pi, (items, ns_))))
        exps, grads = bs.run([v for _, _, v in groups], grads=True)
        for (n, ops, v), e, g in zip(groups, exps, grads):
            for i in range(v.shape[0]):
                re, rg = oracle_item(n, ops, v[i], terms)
                assert abs(e[i, 0] - re) < vtol, (n, i)
                np.testing.assert_allclose(g[i], rg, atol=gtol, err_msg=f"n={n} item={i}")


def test_graph_replay_is_deterministic():
    n = 13
    ops, nslots = encoded_hea(n, 3, seed=1)
    v = np.random.default_rng(1).uniform(-np.pi, np.pi, (16, nslots))
    with BatchSession("c64", grads=True) as bs:
        bs.add_group(n, ops, [(1.0, "Z", [0])], 16, nslots)
        bs.add_group(10, encoded_hea(10, 3, seed=2)[0], [(1.0, "Z", [0])], 4, None)
        v2 = np.random.default_rng(2).uniform(-np.pi, np.pi, (4, bs.groups[1][2]))
        runs = [bs.run([v, v2], grads=True) for _ in range(3)]  # direct, capture + replay, replay
        info = bs.info()
    assert info["graph_ready"][1]
    assert info["kernels_per_run"][1] > 0
    for e, g in runs[1:]:
        for a, b in zip(e + g, runs[0][0] + runs[0][1]):
            assert np.array_equal(a, b)


def test_no_graph_matches_graph():
    n = 12
    ops, nslots = encoded_hea(n, 2, seed=3)
    v = np.random.default_rng(3).uniform(-np.pi, np.pi, (8, nslots))
    out = []
    for graph in (True, False):
        with BatchSession("c64", grads=True, graph=graph) as bs:
            bs.add_group(n, ops, [(1.0, "Z", [0])], 8, nslots)
            for _ in range(3):
                e, g = bs.run([v], grads=True)
            out.append((e[0], g[0]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("n", [9, 13])
def test_weighted_observables(n):
    ops, nslots = encoded_hea(n, 2, seed=n)
    obs = [[(1.0, "Z", [q])] for q in range(n)]
    rng = np.random.default_rng(n)
    items = 4
    v = rng.uniform(-np.pi, np.pi, (items, nslots))
    w = rng.normal(size=(items, n))
    with BatchSession("c128", grads=True) as bs:
        bs.add_group(n, ops, obs, items, nslots)
        e = bs.run([v])
        e2, g = bs.run([v], grads=True, weights=[w])
    np.testing.assert_array_equal(e[0], e2[0])
    for i in range(items):
        psi = oracle.simulate(n, gradients.bind(ops, v[i]))
        for q in range(n):
            assert abs(e[0][i, q] - oracle.expect_pauli(psi, "Z", [q])) < 1e-12
        terms = [(float(w[i, q]), "Z", [q]) for q in range(n)]
        _, rg = oracle_item(n, ops, v[i], terms)
        np.testing.assert_allclose(g[0][i], rg, atol=1e-10)


def test_phase_gates_and_forward_only():
    """rx/p/cp/rzz slots bound on the device; gradients against finite
    differences of the oracle."""
    from test_batch_host import mixed_circuit

    n = 7
    ops, nslots = mixed_circuit(n, seed=3)
    terms = [(1.0, "Z", [0]), (-0.7, "ZZ", [1, 2]), (0.3, "Y", [3]), (0.2, "XZ", [4, 5])]
    v = np.random.default_rng(9).uniform(-np.pi, np.pi, (3, nslots))
    v[0, ::2] = np.pi
    with BatchSession("c128", grads=True) as bs:
        bs.add_group(n, ops, terms, 3, nslots)
        e, g = bs.run([v], grads=True)
    h = 1e-6
    for i in range(3):
        assert abs(e[0][i, 0] - oracle.energy(n, gradients.bind(ops, v[i]), terms)) < 1e-12
        fd = np.zeros(nslots)
        for k in range(nslots):
            ev = []
            for sh in (h, -h):
                w = v[i].copy()
                w[k] += sh
                ev.append(oracle.energy(n, gradients.bind(ops, w), terms))
            fd[k] = (ev[0] - ev[1]) / (2 * h)
        np.testing.assert_allclose(g[0][i], fd, atol=1e-7)
