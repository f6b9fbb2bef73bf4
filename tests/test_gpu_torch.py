"""The torch binding of the batched engine on the GPU: QuantumLayer (shared
weights + per-sample inputs, one observable: Jacobian from the forward run)
and the TorchTransformer.execute drop-in (<Z_i> of every qubit: weighted
adjoint run in backward, Parameter and ParameterExpression angles), both
against the oracle."""

import numpy as np
import pytest
import torch

import oracle
from pyquafu_gb300 import gradients, workloads
from pyquafu_gb300.interface import QuantumLayer, TorchTransformer

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("c128", 1e-10), ("c64", 2e-5)])
def test_quantum_layer_mse_gradient(precision, tol):
    n, layers, batch = 8, 2, 12
    ops, w0, x, y = workloads.qnn_batch(batch=batch, n=n, layers=layers, seed=1)
    nw = 2 * n * layers
    layer = QuantumLayer(n, ops, [(1.0, "Z", [0])], np.arange(nw), nw + np.arange(n), init=w0, precision=precision)
    xt = torch.tensor(x)
    out = layer(xt)
    loss = torch.mean((out[:, 0] - torch.tensor(y)) ** 2)
    loss.backward()
    e_ref = np.zeros(batch)
    g_ref = np.zeros(nw)
    for b in range(batch):
        v = np.concatenate([w0, x[b]])
        bound = gradients.bind(ops, v)
        psi = oracle.simulate(n, bound)
        e_ref[b] = oracle.expect_pauli(psi, "Z", [0])
        g = oracle.grad_adjoint(n, bound, [o.slot for o in bound], [(1.0, "Z", [0])])
        g_ref += 2.0 * (e_ref[b] - y[b]) / batch * g[:nw]
    np.testing.assert_allclose(out[:, 0].detach().numpy(), e_ref, atol=tol)
    np.testing.assert_allclose(layer.weight.grad.numpy(), g_ref, atol=tol)


def test_transformer_execute_dropin():
    n, batch = 6, 5
    ops, _ = workloads.hea(n, 2, seed=3)
    circ = workloads.ProtoCircuit(n, ops, parameters=True)
    nvar = len(circ.variables)
    rng = np.random.default_rng(3)
    params = torch.tensor(rng.uniform(0, 2 * np.pi, (batch, nvar)), requires_grad=True)
    out = TorchTransformer.execute(circ, params, method="adjoint", precision="c128")
    go = torch.tensor(rng.normal(size=(batch, n)))
    (out * go).sum().backward()
    for b in range(batch):
        bound = gradients.bind(ops, params[b].detach().numpy())
        psi = oracle.simulate(n, bound)
        for q in range(n):
            assert abs(out[b, q].item() - oracle.expect_pauli(psi, "Z", [q])) < 1e-12
        terms = [(float(go[b, q]), "Z", [q]) for q in range(n)]
        g = oracle.grad_adjoint(n, bound, [o.slot for o in bound], terms)
        np.testing.assert_allclose(params.grad[b].numpy(), g, atol=1e-10)


def test_batched_param_shift_matches_adjoint():
    from pyquafu_gb300 import gradients

    n, batch = 7, 3
    ops, _ = workloads.hea(n, 2, seed=5)
    slots = max(o.slot for o in ops) + 1
    rng = np.random.default_rng(5)
    v = rng.uniform(0, 2 * np.pi, (batch, slots))
    obs = [[(1.0, "Z", [q])] for q in range(n)]
    e, jac = gradients.jacobian_param_shift(n, ops, obs, v, "c128", chunk_items=20)
    assert jac.shape == (batch, n, slots)
    for b in range(batch):
        bound = gradients.bind(ops, v[b])
        psi = oracle.simulate(n, bound)
        for q in (0, 3, 6):
            g = oracle.grad_adjoint(n, bound, [o.slot for o in bound], [(1.0, "Z", [q])])
            np.testing.assert_allclose(jac[b, q], g, atol=1e-10)
            assert abs(e[b, q] - oracle.expect_pauli(psi, "Z", [q])) < 1e-12
    circ = workloads.ProtoCircuit(n, ops, parameters=True)
    params = torch.tensor(v, requires_grad=True)
    go = torch.tensor(rng.normal(size=(batch, n)))
    (TorchTransformer.execute(circ, params, method="param_shift", precision="c128") * go).sum().backward()
    g_ps = params.grad.clone()
    params.grad = None
    (TorchTransformer.execute(circ, params, method="adjoint", precision="c128") * go).sum().backward()
    np.testing.assert_allclose(g_ps.numpy(), params.grad.numpy(), atol=1e-10)


def test_transformer_execute_parameter_expressions():
    """Angles given as ParameterExpressions of the circuit's variables
    (quantum_circuit.py:285-297 chain rule): outputs and the vector-Jacobian
    product against the oracle's adjoint per gate slot, chained by hand."""
    import test_interface_host as tih

    circ, ops = tih.expression_circuit()
    rng = np.random.default_rng(11)
    batch = 4
    params = torch.tensor(rng.uniform(-2, 2, (batch, 2)), requires_grad=True)
    out = TorchTransformer.execute(circ, params, method="adjoint", precision="c128")
    go = torch.tensor(rng.normal(size=(batch, 2)))
    (out * go).sum().backward()
    for b in range(batch):
        t0, t1 = params[b].detach().numpy()
        angles = [t0, 2 * t1 + np.sin(t0), t1, t0 * t1]
        gates = [o for o in ops]
        for gi, sl in ((0, 0), (2, 1), (3, 2), (4, 3)):
            gates[gi] = type(ops[gi])(ops[gi].name, ops[gi].kind, ops[gi].qubits, 0, (angles[sl],), slot=sl)
        psi = oracle.simulate(2, gates)
        for q in range(2):
            assert abs(out[b, q].item() - oracle.expect_pauli(psi, "Z", [q])) < 1e-12
        terms = [(float(go[b, q]), "Z", [q]) for q in range(2)]
        gs = oracle.grad_adjoint(2, gates, [o.slot for o in gates], terms)
        d0 = gs[0] + gs[1] * np.cos(t0) + gs[3] * t1
        d1 = 2 * gs[1] + gs[2] + gs[3] * t0
        np.testing.assert_allclose(params.grad[b].numpy(), [d0, d1], atol=1e-10)
