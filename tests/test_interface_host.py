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


def test_parameter_expressions_are_refused():
    class ParameterExpression:
        def __float__(self):
            return 0.5

    ops = [ir.Op("ry", ir.OP_RY, (0,), 0, (0.1,), slot=0)]
    circ = workloads.ProtoCircuit(1, ops, parameters=True)
    circ.gates[0].paras[0] = ParameterExpression()
    circ.gates[0]._paras[0] = circ.gates[0].paras[0]
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
