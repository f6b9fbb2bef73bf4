"""The bench.py JSON contract: the reference arm on the CPU (host cores,
oracle port) and, on a GPU, the engine arm's line with every key the
contract names (roofline, e2e, cpu_baseline, clocks, gpu_launches), on a
20-qubit instance of the benchmark circuit."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"}


def run_bench(args, qubits):
    env = dict(os.environ, QFVM_BENCH_QUBITS=str(qubits))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       cwd=ROOT, env=env, timeout=1200)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = run_bench(["--impl", "reference", "--steps", "2", "--warmup", "1"], 16)
    assert BASE_KEYS <= set(d)
    assert d["impl"] == "reference" and d["metric"] == "statevector_gbps" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["qubits"] == 16


@pytest.mark.gpu
def test_engine_arm_line():
    d = run_bench(["--steps", "2", "--warmup", "3", "--no-autotune", "--skip-batch", "--skip-adjoint",
                   "--skip-variants", "--cpu-seconds", "1"], 20)
    assert BASE_KEYS | {"roofline", "clocks", "gpu_launches"} <= set(d)
    rf = d["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(rf)
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-3
    e2e = d["e2e"]
    assert e2e["h2d_bytes_per_step"] == 16 * 2 ** 20 and e2e["d2h_bytes_per_step"] == 16 * 2 ** 20
    assert d["gpu_launches"] > 0 and d["specialised"]["passes"] == d["specialised"]["of"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    # the same workload description as the reference arm, and the error of
    # the result against the oracle
    ref = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "1"], 20)
    assert d["config"] == ref["config"]
    assert d["max_abs_err_vs_oracle"] <= 1e-12
    rows = d["rows"]
    assert rows["C2_30q"][d["engine"]["precision"]]["err"] <= 1e-12
    c1 = rows["C1_20q_4096shots"]
    assert c1["sample_mismatches"] == 0 and c1["err"] <= 1e-12


FORKED_ORACLE_CHECK = """
import os, sys
import numpy as np
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import bench
import oracle
n = 14
ops = bench.workload(n)
run = bench.OracleRun(n, ops)
psi, zz, idx, secs, scan_s = run.result()
ref = oracle.simulate(n, ops)
assert np.array_equal(psi, ref)
assert abs(zz - oracle.expect_pauli(ref, "ZZ", [0, 1])) <= 1e-15
assert np.array_equal(idx, oracle.sample_indices(ref, run.u))
assert secs >= 0 and scan_s >= 0
print("ok")
"""


def test_forked_oracle_run():
    """The bench's oracle run in a child forked before any GPU call: the
    final state in the shared mapping, <Z0 Z1> and the indices of the seeded
    shots equal the oracle's own (a 14-qubit instance of the benchmark
    circuit).  It runs in a fresh interpreter, as in the bench: the fork must
    come before the process's first OpenMP region, since the oracle's OpenMP
    runtime does not carry its thread pool across a fork, and this test
    process has run the oracle already."""
    code = "ROOT = %r\n" % ROOT + FORKED_ORACLE_CHECK
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-2000:]


ABANDONED_ORACLE = """
import os, sys, time
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import bench
n = 24
run = bench.OracleRun(n, bench.workload(n))
print(run.pid, flush=True)
time.sleep(0.5)
raise SystemExit(3)
"""


def test_bench_exit_ends_the_oracle_child():
    """A bench that stops before waiting for the oracle run (an exception in
    the GPU rows) ends its child instead of leaving it computing."""
    code = "ROOT = %r\n" % ROOT + ABANDONED_ORACLE
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 3, r.stderr[-2000:]
    pid = int(r.stdout.split()[0])
    with pytest.raises(ProcessLookupError):
        os.kill(pid, 0)
