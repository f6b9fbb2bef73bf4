"""Generate golden fixtures from the reference implementation itself.

Runs pyquafu (imported from the reference tree) on its own qfvm CPU module
(built by oracle/build_ref.sh from the unmodified src/qfvm/qfvm.cpp) and
records, for seeded circuits built with pyquafu's QuantumCircuit API:

  * the packed gate list read from each circuit by pyquafu_gb300.ir
  * the reference's final statevector (qfvm.simulate_circuit)
  * the reference's expect_statevec values for a set of Pauli strings
  * single-gate applications (qfvm.applyop_statevec) on random states
  * counts of deterministic circuits (bitstring / cbit conventions)
  * gradients from quafu.algorithms.gradients (adjoint and parameter shift)
  * the calls quafu's own front end (quafu.simulate) makes into qfvm, with
    their arguments and the reference module's return values

Usage (build container only; the reference tree is not on GPU machines):
    ./oracle/build_ref.sh && python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refload  # noqa: E402

from pyquafu_gb300 import ir  # noqa: E402


def op_to_json(o: ir.Op) -> dict:
    d = {"name": o.name, "kind": o.kind, "qubits": list(o.qubits), "ncontrols": o.ncontrols,
         "params": list(o.params), "slot": o.slot}
    if o.matrix is not None:
        m = np.asarray(o.matrix, dtype=np.complex128)
        d["matrix"] = [m.real.tolist(), m.imag.tolist()]
    if o.qbits or o.cbits:
        d["qbits"], d["cbits"] = list(o.qbits), list(o.cbits)
    if o.kind == ir.OP_CIF:
        d["condition"] = o.condition
        d["body"] = [op_to_json(b) for b in o.body]
    return d


def build_all_gates_circuit(QuantumCircuit, eg, n, layers, seed):
    """Every gate family pyquafu offers, on random qubits."""
    rng = np.random.default_rng(seed)
    qc = QuantumCircuit(n)
    for _ in range(layers):
        for q in range(n):
            g = int(rng.integers(12))
            th = float(rng.uniform(0, 2 * np.pi))
            if g < 8:
                [qc.h, qc.x, qc.s, qc.t, qc.y, qc.z, qc.sdg, qc.tdg][g](q)
            else:
                [qc.rx, qc.ry, qc.rz, qc.p][g - 8](q, th)
        p = [int(x) for x in rng.permutation(n)]
        th = float(rng.uniform(0, 2 * np.pi))
        qc.cx(p[0], p[1])
        qc.cz(p[1], p[2])
        qc.swap(p[0], p[2])
        qc.rzz(p[1], p[0], th)
        qc.toffoli(p[2], p[0], p[1])
        if n >= 4:
            qc.cp(p[3], p[0], th)
            qc.add_ins(eg.CRYGate(p[0], p[3], th))
            qc.add_ins(eg.CRXGate(p[3], p[1], th))
            qc.add_ins(eg.CRZGate(p[2], p[3], th))
            qc.add_ins(eg.U3Gate(p[2], th, 0.3, 0.7))
            qc.rxx(p[1], p[3], th)
            qc.ryy(p[3], p[2], th)
            qc.iswap(p[0], p[3])
            qc.cy(p[3], p[0])
            qc.sx(p[1])
            qc.sy(p[2])
            qc.w(p[3])
        if n >= 5:
            qc.mcx([p[0], p[1], p[2]], p[4])
            qc.mcz([p[4], p[1]], p[3])
            qc.fredkin(p[4], p[1], p[3])
    return qc


def random_layer_circuit(QuantumCircuit, n, depth, seed, extras):
    """The benchmark generator (pyquafu_gb300.workloads.random_layers) built
    through pyquafu's API."""
    from pyquafu_gb300 import workloads

    ops = workloads.random_layers(n, depth, seed, extras=extras)
    qc = QuantumCircuit(n)
    for o in ops:
        if o.name in ("rx", "ry", "rz"):
            getattr(qc, o.name)(o.qubits[0], o.params[0])
        elif o.name == "rzz":
            qc.rzz(o.qubits[0], o.qubits[1], o.params[0])
        elif o.name == "ccx":
            qc.toffoli(*o.qubits)
        else:
            getattr(qc, o.name)(*o.qubits)
    return qc


PAULI_SETS = [
    ("Z0", None), ("Z0 Z1", None), ("X0", None), ("Y1", None), ("X0 X1", None), ("Y0 Y2", None),
    ("X0 Y1 Z2", None), ("Z1 Z2", None), ("X1 Z0", None), ("Y2 X0", None),
]


class RecordingQfvm:
    """Stands in for quafu.simulators.qfvm while quafu's own front end runs:
    forwards every call to the reference module and, while `calls` is a
    list, records what the front end passed and what it got back."""

    def __init__(self, ref):
        self.ref = ref
        self.calls = None
        self.states = {}

    def _circuit(self, qc):
        circ = ir.read_circuit(qc)
        return {"n": qc.num, "cbits_num": qc.cbits_num, "ops": [op_to_json(o) for o in circ.ops],
                "measures": [list(m) for m in circ.measure_vec]}

    def _state(self, key, psi):
        tag = f"frontend_{len(self.states)}_{key}"
        self.states[tag] = np.array(psi, dtype=np.complex128, copy=True)
        return tag

    def simulate_circuit(self, qc, inputstate=np.array(0, dtype=np.complex128), shots=0):
        rec = None
        if self.calls is not None:
            rec = {"fn": "simulate_circuit", "circuit": self._circuit(qc), "shots": int(shots),
                   "input": self._state("in", inputstate) if np.size(inputstate) else None}
        counts, psi = self.ref.simulate_circuit(qc, inputstate, shots)
        if rec is not None:
            rec["counts"] = {str(k): int(v) for k, v in dict(counts).items()}
            rec["output"] = self._state("out", psi)
            self.calls.append(rec)
        return counts, psi

    def expect_statevec(self, inputstate, paulis):
        res = self.ref.expect_statevec(inputstate, paulis)
        if self.calls is not None:
            self.calls.append({"fn": "expect_statevec", "input": self._state("in", inputstate),
                               "paulis": [[p.paulistr, [int(x) for x in p.pos]] for p in paulis],
                               "result": [float(x) for x in res]})
        return res

    def applyop_statevec(self, op, inputstate):
        return self.ref.applyop_statevec(op, inputstate)

    def sampling_statevec(self, measures, inputstate, shots):
        return self.ref.sampling_statevec(measures, inputstate, shots)

    def simulate_circuit_clifford(self, qc, shots):
        return self.ref.simulate_circuit_clifford(qc, shots)


def main():
    ref = refload.load_ref_qfvm()
    recorder = RecordingQfvm(ref)
    refload.load(recorder)  # quafu imports its qfvm functions from the recorder
    from quafu import QuantumCircuit
    import quafu.elements.element_gates as eg
    from quafu.algorithms.hamiltonian import Hamiltonian, PauliOp
    from quafu.elements import Parameter
    out_cases = []
    states = {}

    def record(tag, qc, n, psi_in=None, paulis=None):
        circ = ir.read_circuit(qc)
        inp = np.zeros(0, dtype=np.complex128) if psi_in is None else psi_in.copy()
        _, psi = ref.simulate_circuit(qc, inp, 0)
        case = {"tag": tag, "n": n, "ops": [op_to_json(o) for o in circ.ops], "final_measure": circ.final_measure,
                "has_input": psi_in is not None}
        states[f"{tag}__out"] = np.asarray(psi, dtype=np.complex128)
        if psi_in is not None:
            states[f"{tag}__in"] = psi_in
        if paulis:
            terms = [p for p in paulis if max(int(x[1:]) for x in p.split()) < n]
            pobjs = [PauliOp(p) for p in terms]
            case["paulis"] = [[po.paulistr, list(po.pos)] for po in pobjs]
            case["expect"] = list(ref.expect_statevec(np.asarray(psi), pobjs))
        out_cases.append(case)

    for n, layers, seed in [(3, 4, 11), (5, 4, 12), (7, 5, 13), (9, 4, 14), (12, 3, 15)]:
        qc = build_all_gates_circuit(QuantumCircuit, eg, n, layers, seed)
        record(f"allgates_n{n}", qc, n, paulis=[p for p, _ in PAULI_SETS])
    qc = random_layer_circuit(QuantumCircuit, 10, 20, 0, extras=False)
    record("layers_n10_d20", qc, 10, paulis=["Z0 Z1", "X3", "Y4 Z7"])
    qc = random_layer_circuit(QuantumCircuit, 14, 12, 1, extras=True)
    record("layers_extras_n14_d12", qc, 14, paulis=["Z0 Z1", "X13", "Y2 X9"])
    qc = random_layer_circuit(QuantumCircuit, 16, 10, 2, extras=True)
    record("layers_extras_n16_d10", qc, 16, paulis=["Z0 Z1", "X15 X0"])
    rng = np.random.default_rng(99)
    psi_in = rng.normal(size=64) + 1j * rng.normal(size=64)
    psi_in /= np.linalg.norm(psi_in)
    qc = build_all_gates_circuit(QuantumCircuit, eg, 6, 2, 16)
    record("input_state_n6", qc, 6, psi_in=psi_in.astype(np.complex128), paulis=["Z0", "X5 Y0"])

    # single-gate applications (applyop_statevec) on random states
    apply_cases = []
    rng = np.random.default_rng(7)
    gates = [eg.HGate(2), eg.XGate(0), eg.YGate(3), eg.ZGate(1), eg.SGate(4), eg.SdgGate(0), eg.TGate(2),
             eg.TdgGate(3), eg.RXGate(1, 0.7), eg.RYGate(4, 1.9), eg.RZGate(0, 2.3), eg.PhaseGate(2, 0.4),
             eg.CXGate(0, 3), eg.CXGate(4, 1), eg.CZGate(2, 0), eg.CPGate(3, 1, 1.1), eg.ToffoliGate(0, 4, 2),
             eg.RZZGate(1, 3, 0.9), eg.SwapGate(0, 4), eg.ISwapGate(3, 1), eg.U3Gate(2, 0.5, 1.5, 2.5),
             eg.CRYGate(4, 0, 0.8), eg.MCXGate([1, 2, 3], 0), eg.RXXGate(0, 2, 1.3), eg.SXGate(4),
             eg.FredkinGate(2, 0, 4), eg.CYGate(1, 4), eg.MCZGate([0, 1], 4)]
    for i, g in enumerate(gates):
        psi = rng.normal(size=32) + 1j * rng.normal(size=32)
        psi = (psi / np.linalg.norm(psi)).astype(np.complex128)
        before = psi.copy()
        after = np.asarray(ref.applyop_statevec(g, psi.copy()))
        o = ir.read_op(g)
        apply_cases.append({"tag": f"apply_{i}_{o.name}", "op": op_to_json(o)})
        states[f"apply_{i}__in"] = before
        states[f"apply_{i}__out"] = after

    # deterministic counts: simulate_circuit keys are int(bitstring, 2) with
    # cbit 0 the most significant character (qfvm.cpp:93-97)
    count_cases = []

    def counts_case(tag, qc, shots=50):
        counts, psi = ref.simulate_circuit(qc, np.zeros(0, dtype=np.complex128), shots)
        circ = ir.read_circuit(qc)
        count_cases.append({"tag": tag, "n": qc.num, "ops": [op_to_json(o) for o in circ.ops],
                            "measures": [list(m) for m in circ.measure_vec], "shots": shots,
                            "counts": {str(k): int(v) for k, v in dict(counts).items()}})

    qc = QuantumCircuit(2, 2)
    qc.x(0)
    qc.x(1)
    qc.measure([0, 1])
    counts_case("x_x_measure", qc)
    qc = QuantumCircuit(4, 4)
    qc.x(0)
    qc.x(1)
    qc.measure([1, 2], [1, 0])
    qc.measure([3, 0], [2, 3])
    counts_case("any_cbit", qc)
    qc = QuantumCircuit(3, 3)
    qc.x(0)
    qc.cx(0, 2)
    qc.measure([0, 1, 2], [2, 1, 0])
    counts_case("reversed_cbits", qc)
    qc = QuantumCircuit(5, 2)
    qc.x(3)
    qc.x(1)
    qc.measure([3, 1], [0, 1])
    counts_case("partial_measure", qc)

    # circuits with operations after a measurement: the per-shot branch
    # (qfvm.cpp:104-133), deterministic outcomes; the circuits are those of
    # tests/quafu/simulator/classic_test.py:25-93 (the input-state case,
    # classic_test.py:176-185, trips the reference's adopted-buffer bug and is
    # left out)
    mid_cases = []

    def mid_case(tag, qc, shots=10):
        counts, psi = ref.simulate_circuit(qc, np.zeros(0, dtype=np.complex128), shots)
        circ = ir.read_circuit(qc)
        mid_cases.append({"tag": tag, "n": qc.num, "cbits": qc.cbits_num, "ops": [op_to_json(o) for o in circ.ops],
                          "final_measure": circ.final_measure, "shots": shots,
                          "counts": {str(k): int(v) for k, v in dict(counts).items()}})
        states[f"mid_{tag}"] = np.asarray(psi)

    qc = QuantumCircuit(2, 2)
    qc.x(0)
    qc.measure([0], [0])
    with qc.cif([0], 1):
        qc.x(1)
    qc.measure([1], [1])
    mid_case("cif_true", qc)
    qc = QuantumCircuit(2)
    qc.measure([0], [0])
    with qc.cif([0], 1):
        qc.x(1)
    qc.measure([1], [1])
    mid_case("cif_false", qc)
    qc = QuantumCircuit(3, 3)
    qc.x(0)
    qc.cx(0, 1)
    qc.measure([0, 1], [0, 1])
    with qc.cif([0, 1], 3):
        qc.x(2)
    qc.measure([2], [2])
    mid_case("cif_list_true", qc)
    qc = QuantumCircuit(3)
    qc.x(0)
    qc.cx(0, 1)
    qc.measure([0, 1], [0, 1])
    for cond in (0, 1, 2, 4):
        with qc.cif([0, 1], cond):
            qc.x(2)
    qc.measure([2], [2])
    mid_case("cif_list_false", qc)
    qc = QuantumCircuit(2)
    qc.x(0)
    qc.measure([0], [0])
    qc.reset([0])
    qc.measure([0], [1])
    mid_case("single_reset", qc)
    qc = QuantumCircuit(4)
    qc.x(0)
    qc.cx(0, 1)
    qc.measure([0, 1], [0, 1])
    qc.reset([0, 1])
    qc.measure([0, 1], [2, 3])
    mid_case("multi_reset", qc)
    qc = QuantumCircuit(3, 3)
    qc.x(1)
    qc.x(2)
    qc.cx(2, 0)
    qc.reset([1])
    qc.x(0)
    qc.measure([0], [0])
    with qc.cif([0], 0):  # the reference reads no parameterised gate inside a cif
        qc.x(1)
        qc.h(2)
    qc.measure([1], [1])
    mid_case("reset_then_cif", qc, shots=1)

    # noisy trajectories (NoiseSVSimulator.run, simulator.py:174-203) with
    # numpy's generator seeded: per shot the reference draws one number per
    # unitary channel, then one per Kraus channel, from np.random (replayable);
    # its final sample uses the engine's own generator, so counts are recorded
    # only for circuits whose final state is a basis state.  psi=None: the
    # reference's `if not psi` rejects numpy arrays on this numpy.
    from quafu.elements.noise import AmplitudeDamping, BitFlip, Decoherence, Dephasing, Depolarizing
    from quafu.simulators.simulator import NoiseSVSimulator

    noise_cases = []

    def noise_case(tag, qc, terms, shots, seed, with_counts):
        hamil = Hamiltonian.from_pauli_list(terms) if terms else None
        np.random.seed(seed)
        res = NoiseSVSimulator().run(qc, psi=None, shots=shots, hamiltonian=hamil)
        ops = []
        for ins in qc.instructions:
            o = ir.read_noisy_op(ins)
            if o is not None and o.kind != ir.OP_MEASURE:
                ops.append(o)
        case = {"tag": tag, "n": qc.num, "ops": [op_to_json(o) for o in ops], "shots": shots, "seed": seed,
                "measures": [[int(q), int(c)] for q, c in qc.measures.items()],
                "terms": [[t[0], float(t[1])] for t in terms],
                "pauli_expects": [float(v) for v in res["pauli_expects"]]}
        if with_counts:
            case["counts"] = {str(k): int(v) for k, v in dict(res["counts"]).items()}
        noise_cases.append(case)

    qc = QuantumCircuit(3)
    qc << eg.HGate(0) << eg.CXGate(0, 1) << Depolarizing(1, 0.3) << BitFlip(2, 0.4)
    qc << AmplitudeDamping(0, 0.25) << eg.RYGate(2, 0.7) << Dephasing(0, 0.2) << Decoherence(1, 2.0, 30.0, 20.0)
    qc << eg.CXGate(1, 2) << AmplitudeDamping(2, 0.5)
    qc.measure([0, 1, 2])
    noise_case("mixed_channels", qc, [("Z0", 1.0), ("X1 Z2", 0.5), ("Y0 Y1", -0.3), ("Z2", 0.8)], 40, 7, False)
    qc = QuantumCircuit(2)
    qc << eg.XGate(0) << BitFlip(1, 0.5) << Depolarizing(0, 0.6)
    qc.measure([0, 1])
    noise_case("basis_flips", qc, [("Z0", 1.0), ("Z1", 1.0)], 30, 11, True)

    # sampling_statevec on basis states: {bitstring: count}
    sampling_cases = []
    for idx, meas in [(5, {0: 0, 1: 1, 2: 2, 3: 3}), (6, {2: 0, 1: 1}), (9, {3: 1, 0: 0}), (12, {3: 0, 2: 1, 0: 2})]:
        psi = np.zeros(16, dtype=np.complex128)
        psi[idx] = 1.0
        counts = ref.sampling_statevec(meas, psi.copy(), 20)
        sampling_cases.append({"index": idx, "n": 4, "measures": [[int(k), int(v)] for k, v in meas.items()],
                               "shots": 20, "counts": {str(k): int(v) for k, v in dict(counts).items()}})

    # gradients through quafu.algorithms.gradients on the reference engine
    from quafu.algorithms.gradients.gradiant import grad_adjoint, grad_para_shift

    grad_cases = []

    def grad_case(tag, n, build, pauli_list):
        qc = build()
        pg = qc.get_parameter_grads()  # registers the Parameters (quantum_circuit.py:256-283)
        ham = Hamiltonian.from_pauli_list(pauli_list)
        adj = grad_adjoint(qc, ham)
        ps = grad_para_shift(qc, ham)
        res = sum(__import__("quafu").simulate(qc, hamiltonian=ham)["pauli_expects"])
        circ = ir.read_circuit(qc)
        ops = circ.ops
        pgates = set()
        assembly = []
        for var, items in pg.items():
            row = []
            for (i, j), coeff in items:
                pgates.add(i)
                row.append([int(i), float(coeff)])
            assembly.append(row)
        for i, o in enumerate(ops):
            o.slot = i if i in pgates else -1  # one slot per parameterised gate
        grad_cases.append({"tag": tag, "n": n, "ops": [op_to_json(o) for o in ops], "assembly": assembly,
                           "terms": [[float(np.real(c)), *_split(p)] for p, c in pauli_list],
                           "energy": float(res), "adjoint": [float(x) for x in adj],
                           "param_shift": [float(x) for x in ps]})

    def _split(p):
        parts = p.split()
        return ["".join(x[0] for x in parts), [int(x[1:]) for x in parts]]

    def ref_test_gradient():
        # the circuit of tests/quafu/algorithms/varational_test.py:68-83
        from quafu.elements.element_gates import CXGate, HGate, RYGate

        pq = QuantumCircuit(4)
        theta = [Parameter("theta_%d" % (i), i + 1) for i in range(4)]
        for i in range(4):
            pq << HGate(i)
        for i in range(3):
            pq << CXGate(i, i + 1)
        for i in range(4):
            pq << RYGate(i, theta[i])
        for i in range(3):
            pq << CXGate(i, i + 1)
        for i in range(4):
            pq << RYGate(i, theta[i])
        pq << RYGate(2, theta[0] * theta[1] - 3 * theta[0])
        return pq

    grad_case("ref_test_gradient", 4, ref_test_gradient, [("X1 X2", 1.0), ("Z0 Z3", 1.0)])

    def vqe4():
        qc = QuantumCircuit(4)
        th = [Parameter(f"t{i}", v) for i, v in enumerate([0.3, 1.2, -0.7, 2.1])]
        qc.h(0)
        qc.h(1)
        qc.cx(0, 1)
        qc.ry(0, th[0])
        qc.ry(1, th[1])
        qc.cx(1, 2)
        qc.ry(2, th[2])
        qc.rx(3, th[3])
        qc.cx(2, 3)
        qc.rz(3, th[0])
        return qc

    grad_case("vqe4", 4, vqe4, [("X1 X2", 1.0), ("Z0 Z3", 1.0), ("Y0 Y1", 0.5)])

    def hea(n, layers, seed):
        def b():
            rng = np.random.default_rng(seed)
            qc = QuantumCircuit(n)
            k = 0
            for _ in range(layers):
                for q in range(n):
                    qc.ry(q, Parameter(f"p{k}", float(rng.uniform(0, 2 * np.pi))))
                    k += 1
                for q in range(n):
                    qc.rz(q, Parameter(f"p{k}", float(rng.uniform(0, 2 * np.pi))))
                    k += 1
                for q in range(n - 1):
                    qc.cx(q, q + 1)
            return qc
        return b

    rng = np.random.default_rng(5)
    n = 6
    terms = [(f"Z{i} Z{i+1}", float(rng.normal())) for i in range(n - 1)] + [(f"X{i}", float(rng.normal())) for i in range(n)]
    grad_case("hea6_l3", n, hea(n, 3, 21), terms)

    # quafu's own front end (quafu.simulate -> SVSimulator.run,
    # simulator.py:90-145) over the recording module: the calls it makes into
    # qfvm and what the reference module returned for them
    import quafu

    recorder.calls = []
    qc = QuantumCircuit(4, 4)
    qc.x(0)
    qc.x(2)
    qc.cx(2, 3)
    qc.measure([0, 1, 2, 3], [3, 2, 1, 0])
    quafu.simulate(qc, shots=64)
    qc = random_layer_circuit(QuantumCircuit, 10, 12, 4, extras=True)
    ham = Hamiltonian.from_pauli_list([("Z0 Z1", 0.7), ("X3 Y4", -0.4), ("Z9", 1.1)])
    quafu.simulate(qc, hamiltonian=ham)
    rng = np.random.default_rng(41)
    psi0 = rng.normal(size=1 << 6) + 1j * rng.normal(size=1 << 6)
    psi0 = (psi0 / np.linalg.norm(psi0)).astype(np.complex128)
    qc = build_all_gates_circuit(QuantumCircuit, eg, 6, 2, 42)
    quafu.simulate(qc, psi=psi0.copy(), hamiltonian=Hamiltonian.from_pauli_list([("X0 Z5", 1.0), ("Y2", 0.5)]))
    frontend_calls = recorder.calls
    recorder.calls = None
    states.update(recorder.states)

    meta = {"cases": out_cases, "apply": apply_cases, "counts": count_cases, "sampling": sampling_cases,
            "gradients": grad_cases, "mid_circuit": mid_cases, "noise": noise_cases, "frontend": frontend_calls,
            "generator": "tests/golden/make_golden.py (reference qfvm.cpp via oracle/build_ref.sh)"}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f)
    np.savez_compressed(os.path.join(HERE, "golden_states.npz"), **states)
    print(f"{len(out_cases)} circuits, {len(apply_cases)} single gates, {len(count_cases)} count cases, "
          f"{len(sampling_cases)} sampling cases, {len(grad_cases)} gradient cases")


if __name__ == "__main__":
    main()
