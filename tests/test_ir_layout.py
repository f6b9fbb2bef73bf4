"""Circuit reader and packed layout (host logic, no GPU)."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from pyquafu_gb300 import ir, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reader_on_protocol_objects():
    ops = workloads.random_layers(6, 3, seed=1, extras=True, extra_rate=1.0)
    pc = workloads.as_protocol(6, ops, measures=[(0, 0), (3, 1)])
    circ = ir.read_circuit(pc)
    assert circ.num_qubits == 6 and circ.final_measure
    assert circ.measure_vec == [(0, 0), (3, 1)]
    got = [o for o in circ.ops if o.is_gate]
    assert [(o.name, o.qubits, o.params) for o in got] == [(o.name, o.qubits, o.params) for o in ops]
    swap = [o for o in got if o.name == "swap"][0]
    assert swap.kind == ir.OP_MATRIX and swap.matrix.shape == (4, 4)


def test_measure_then_gate_clears_final_measure():
    class M:
        name = "measure"
        qbits = [0]
        cbits = [0]

    class X:
        name = "X"
        pos = [1]
        _paras = []

    class C:
        num = 2
        cbits_num = 2
        instructions = [M(), X()]

    assert not ir.read_circuit(C()).final_measure


def test_skipped_and_wrapped():
    class B:
        name = "barrier"
        pos = [0, 1]

    class H:
        name = "H"
        pos = [0]
        _paras = []

    class Inner:
        num = 2
        cbits_num = 2
        instructions = [H()]

    class W:
        name = "oracle"
        circuit = Inner()

    class C:
        num = 2
        cbits_num = 2
        instructions = [B(), W(), H()]

    circ = ir.read_circuit(C())
    assert [o.name for o in circ.ops] == ["h", "h"]


def test_validate_rejects_bad_input():
    with pytest.raises(ValueError):
        ir.validate([workloads.named("h", (5,))], 3)
    with pytest.raises(ValueError):
        ir.validate([workloads.named("cx", (1, 1), ncontrols=1)], 3)
    with pytest.raises(ValueError):
        ir.validate([workloads.named("rx", (0,), (float("nan"),))], 3)
    with pytest.raises(ValueError):
        ir.validate([workloads.matrix_gate("u", (0, 1), np.eye(2))], 3)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_op_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "qfvm_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(qfvm_op),"
        " offsetof(qfvm_op, kind), offsetof(qfvm_op, ncontrols), offsetof(qfvm_op, nqubits),"
        " offsetof(qfvm_op, mat_dim), offsetof(qfvm_op, qubits), offsetof(qfvm_op, slot),"
        " offsetof(qfvm_op, params), offsetof(qfvm_op, mat_offset)); return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    d = ir.OP_DTYPE
    assert vals == [d.itemsize, d.fields["kind"][1], d.fields["ncontrols"][1], d.fields["nqubits"][1],
                    d.fields["mat_dim"][1], d.fields["qubits"][1], d.fields["slot"][1], d.fields["params"][1],
                    d.fields["mat_offset"][1]]


def test_pack_matrix_pool():
    ops = [workloads.named("h", (0,)), workloads.matrix_gate("swap", (0, 1), workloads.SWAP),
           workloads.matrix_gate("u", (2,), np.array([[0, 1j], [1j, 0]]))]
    arr, pool = ir.pack(ops)
    assert list(arr["mat_offset"]) == [-1, 0, 16]
    assert list(arr["mat_dim"]) == [0, 4, 2]
    assert pool.size == 20 and pool[17] == 1j
