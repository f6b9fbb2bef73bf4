"""Host side of the torch binding (no GPU): a circuit's Parameter objects map
to engine slots, shared parameters fold into one variable, and the
reference-protocol stand-in reports its variables in first-use order."""

import numpy as np
import pytest

from pyquafu_gb300 import ir, workloads
from pyquafu_gb300.interface import _CircuitBinding


def test_binding_maps_gate_slots_to_variables():
    ops = [ir.Op("ry", ir.OP_RY, (0,), 0, (0.1,), slot=0), workloads.named("h", (1,)),
           ir.Op("rz", ir.OP_RZ, (1,), 0, (0.2,), slot=1), ir.Op("rx", ir.OP_RX, (0,), 0, (0.1,), slot=0)]
    circ = workloads.ProtoCircuit(2, ops, parameters=True)
    assert [v.name for v in circ.variables] == ["theta_0", "theta_1"]
    b = _CircuitBinding(circ)
    assert b.n == 2 and b.num_vars == 2
    assert [g.slot for g in b.gates] == [0, -1, 1, 2]
    assert b.var_of_slot.tolist() == [0, 1, 0]
    grads = circ.get_parameter_grads()
    assert grads[circ.variables[0]] == [[(0, 0), 1.0], [(3, 0), 1.0]]


def expression_circuit():
    """ry(theta_0) on 0, rz(2 theta_1 + sin theta_0) on 1, rx(theta_1) on 0,
    ry(theta_0 * theta_1) on 1 (the last two as ParameterExpressions)."""
    ops = [ir.Op("ry", ir.OP_RY, (0,), 0, (0.1,), slot=0), workloads.named("h", (1,)),
           ir.Op("rz", ir.OP_RZ, (1,), 0, (0.2,), slot=1), ir.Op("rx", ir.OP_RX, (0,), 0, (0.3,), slot=1),
           ir.Op("ry", ir.OP_RY, (1,), 0, (0.4,), slot=0), workloads.named("cx", (0, 1), ncontrols=1)]
    circ = workloads.ProtoCircuit(2, ops, parameters=True)
    t0, t1 = circ._vars
    e1 = workloads.ParameterExpression([t1, t0], lambda x: 2 * x[0] + np.sin(x[1]),
                                       lambda x: np.array([2.0, np.cos(x[1])]))
    e2 = workloads.ParameterExpression([t0, t1], lambda x: x[0] * x[1], lambda x: np.array([x[1], x[0]]))
    for gi, e in ((2, e1), (4, e2)):
        circ.gates[gi].paras[0] = e
        circ.gates[gi]._paras[0] = e
    return circ, ops


def test_parameter_expression_slots_and_chain_rule():
    import torch

    circ, _ = expression_circuit()
    b = _CircuitBinding(circ)
    assert b.num_vars == 2 and b.num_slots == 4
    assert [g.slot for g in b.gates] == [0, -1, 1, 2, 3, -1]
    x = torch.tensor([[0.7, -0.4], [1.3, 2.1]], dtype=torch.float64, requires_grad=True)
    v = b.values(x)
    xs = x.detach().numpy()
    want = np.stack([xs[:, 0], 2 * xs[:, 1] + np.sin(xs[:, 0]), xs[:, 1], xs[:, 0] * xs[:, 1]], axis=1)
    np.testing.assert_allclose(v.detach().numpy(), want, atol=1e-15)
    w = torch.tensor([[1.0, 2.0, 3.0, 4.0], [-1.0, 0.5, 0.25, 2.0]], dtype=torch.float64)
    (v * w).sum().backward()
    # d/dtheta_0: w0 + w1 cos(theta_0) + w3 theta_1; d/dtheta_1: 2 w1 + w2 + w3 theta_0
    wn = w.numpy()
    g0 = wn[:, 0] + wn[:, 1] * np.cos(xs[:, 0]) + wn[:, 3] * xs[:, 1]
    g1 = 2 * wn[:, 1] + wn[:, 2] + wn[:, 3] * xs[:, 0]
    np.testing.assert_allclose(x.grad.numpy(), np.stack([g0, g1], axis=1), atol=1e-14)


def test_only_first_angle_may_be_trainable():
    circ = workloads.ProtoCircuit(1, [ir.Op("ry", ir.OP_RY, (0,), 0, (0.1,), slot=0)], parameters=True)
    circ.gates[0].paras = [0.3, circ._vars[0]]
    with pytest.raises(NotImplementedError):
        _CircuitBinding(circ)


def test_workload_shapes():
    g = workloads.uneven_batch(circuits=64, seed=0)
    assert sum(v[1].shape[0] for v in g.values()) == 64
    for n, (ops, vals) in g.items():
        assert vals.shape[1] == 2 * n * 6 + n == max(o.slot for o in ops) + 1
        assert np.all(vals[:, -n:] >= -np.pi) and np.all(vals[:, -n:] <= np.pi)
    ops, w, x, y = workloads.qnn_batch(batch=32, n=16, layers=12)
    assert w.shape == (384,) and x.shape == (32, 16) and set(np.unique(y)) <= {-1.0, 1.0}
    assert max(o.slot for o in ops) + 1 == 400
