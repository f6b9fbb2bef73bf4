"""Benchmark: statevector gate sweeps of a 30-qubit complex128 random circuit.

Workload (seeded, synthetic): 30 qubits, complex128 (16 GiB state), 40 random
layers (one of h/x/s/t/rx/ry/rz per qubit, angles U[0, 2pi), then cx on a
random perfect matching), plus cz/swap/rzz on random pairs and ccx on a
random triple in ~5% of layers; seed 0 (1808 gates).  One step = one full
circuit on the device-resident state.  The state (16 GiB) is far larger than
L2, so no L2 flush is needed between steps.

metric  statevector_gbps: circuit throughput as gate-equivalent bytes, i.e.
        sum over the circuit's gates of 2 * 16 B * (amplitudes the gate must
        touch), divided by the circuit time.  Both arms use the same
        numerator, so the ratio of two lines is a speed ratio.  It is not an
        HBM figure: the engine fuses many gates per pass over the state; the
        HBM figures are `roofline` (the dominant kernel) and `hbm_gbps`
        (every pass's read + write of the state over the circuit time).
e2e     the same metric through pyquafu_gb300.qfvm.simulate_circuit (the
        reference's API) with the input state in pinned host memory: H2D of
        the state, the run, and D2H of the result are inside the timed region.

The default arithmetic is complex128 storage with float-pair arithmetic
(`c128_ds`, the engine's default for complex128 work); IEEE FP64 (`c128`)
and complex64 (`c64`) are reported as variants.  After the timed rows, the
final state of every variant is compared with the oracle (the CPU
restatement of the reference's FP64 path, run on the host cores), and the
24-qubit adjoint gradients with the oracle's adjoint (--skip-oracle-check
skips both).

--impl reference times the reference algorithm on the host cores instead (the
CPU restatement in oracle/, OpenMP over all cores) on a bounded sample of the
same circuit and state size: each step applies a stride of the circuit's
gates, so the sample covers the whole gate mix.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = int(os.environ.get("QFVM_BENCH_QUBITS", "30"))
DEPTH = 40
SEED = 0
S128 = 16
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
# DRAM bytes per launch of the one-state tile pass, from ncu captures of the
# 26-qubit case of this generator (dram__bytes_read + dram__bytes_write for
# 2^26 amplitudes), scaled by the amplitudes a launch processes (traffic grows
# in proportion: each pass reads and writes every amplitude once)
TRAFFIC_PER_AMP = {"c128": 2.086e9 / 2 ** 26, "c128_ds": 2.087e9 / 2 ** 26}
# the C2 random circuit with the arithmetic the engine defaults to
DEFAULT_PRECISION = "c128_ds"
ORACLE_FLAGS = "gcc -O2 -fopenmp -ffp-contract=off (oracle/qsv_oracle.c)"


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def workload(n=N_QUBITS, depth=DEPTH, seed=SEED):
    from pyquafu_gb300 import workloads

    return workloads.random_layers(n, depth, seed, extras=True)


def cpu_info():
    """Model name and logical CPU count of the host (for the CPU baselines)."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return {"model": model or "unknown", "cores": os.cpu_count() or 1, "build": ORACLE_FLAGS}


def config_of(n, ops):
    """The workload description both arms print (identical dicts)."""
    return {"workload": f"random_layers_{n}q_c128_depth40_extras", "qubits": n, "depth": DEPTH, "seed": SEED,
            "gates": len(ops), "l2": f"state {16 * 2 ** n / 2 ** 30:g} GiB"
                                      + (" >> L2 (no flush needed)" if 16 * 2 ** n > 4 * 129e6 else "")}


def max_abs_diff(a, b, chunk=1 << 24):
    m = 0.0
    for i in range(0, a.size, chunk):
        m = max(m, float(np.abs(a[i:i + chunk] - b[i:i + chunk]).max()))
    return m


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


STRIDE = 301  # coprime with the gate count: t -> (t * STRIDE) mod gates visits every gate


def strided_gates(ops, start, count):
    """Gate indices start .. start+count-1 of the circuit's strided order: a
    bounded sample that covers the whole gate mix."""
    return [(t * STRIDE) % len(ops) for t in range(start, start + count)]


def cpu_sample(ops, n, seconds=12.0):
    """Time the CPU restatement of the reference (oracle/) on the host cores:
    apply the circuit's gates in strided order to a 2^n complex128 state
    until `seconds` have elapsed; returns (gbps, gates applied, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    oracle.build()
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    gate_bytes = gate_equiv_bytes(ops, n)
    done, bytes_done = 0, 0.0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 <= seconds:
        i = strided_gates(ops, done, 1)[0]
        oracle.apply_op(psi, ops[i])
        bytes_done += gate_bytes[i]
        done += 1
    dt = time.perf_counter() - t0
    return bytes_done / dt / 1e9, done, dt


def gate_equiv_bytes(ops, n, S=S128):
    """Per-gate algorithmic bytes: 2 * S * amplitudes the gate must touch."""
    N = float(2 ** n)
    out = []
    for o in ops:
        amps = N / 2.0 ** o.ncontrols
        if o.name in ("s", "sdg", "t", "tdg", "p", "cp", "z", "cz"):
            amps *= 0.5
        elif o.name == "swap":
            amps *= 0.5
        out.append(2.0 * S * amps)
    return out


def run_reference(args):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    ops = workload()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    n = N_QUBITS
    gb = gate_equiv_bytes(ops, n)
    per_step = max(1, env_int("QFVM_REF_GATES_PER_STEP", 6))
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    pos = 0

    def step():
        nonlocal pos
        b = 0.0
        for i in strided_gates(ops, pos, per_step):
            oracle.apply_op(psi, ops[i])
            b += gb[i]
        pos += per_step
        return b

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    tot = 0.0
    for _ in range(args.steps):
        tot += step()
    dt = time.perf_counter() - t0
    v = tot / dt / 1e9
    info = cpu_info()
    sample = (f"{per_step} gates per step in strided order (gate t*{STRIDE} mod {len(ops)}), {args.steps} steps "
              f"after {args.warmup} warm-up steps, on a {16 * 2 ** n / 2 ** 30:g} GiB complex128 state "
              f"(oracle/qsv_oracle.c, OpenMP {cores} threads, {info['model']})")
    line = {"impl": "reference", "metric": "statevector_gbps", "value": round(v, 3), "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_of(n, ops),
            "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                             "sample": sample, "cpu": info},
            "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


S_OF = {"c128": 16, "c128_ds": 16, "c64": 8}
POLICY_OF = {"c128": "P64", "c128_ds": "PDS", "c64": "P32"}


def kernel_name(precision, n, specialised=False):
    """The one-state pass kernel a plan of n qubits runs (shape as resolved
    by the engine: tuned or built-in): the circuit-specialised PTX kernel
    `qsv_tile_pass_*` when the plan's passes were specialised, else the
    interpreting k_pass instance."""
    from pyquafu_gb300 import autotune

    t, r = autotune.current(precision, 0, n)
    if specialised:
        name = {"c128": "qsv_tile_pass_c128", "c128_ds": "qsv_tile_pass_ds", "c64": "qsv_tile_pass_c64"}[precision]
        return f"{name} (specialised PTX, tile {t}, registers {r})"
    return f"k_pass<{POLICY_OF[precision]},{t},{r}>"


def measure(precision, ops, n, steps, warmup, per_pass=True):
    """Device-resident measurement of one precision: returns a dict."""
    import torch

    from pyquafu_gb300 import _native as nat
    from pyquafu_gb300 import engine

    S = S_OF[precision]
    plan = engine.Plan(n, ops, precision)
    st_plan = plan.stats()
    state = engine.DeviceState(n, precision).set_zero()
    stream = torch.cuda.ExternalStream(state.stream())
    t_first = time.perf_counter()
    for _ in range(warmup):
        plan.run(state)
    torch.cuda.synchronize()
    warm_s = time.perf_counter() - t_first  # includes compiling specialised passes
    specialised = plan.jit_passes(1)
    l0 = nat.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    pass_ms, pass_ty = [], []
    for _ in range(steps):
        if per_pass:
            ms, ty = plan.run_timed(state)
            pass_ms.append(ms)
            pass_ty.append(ty)
        else:
            plan.run(state)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = nat.launch_count() - l0
    ms_step = ev0.elapsed_time(ev1) / steps
    gb = sum(gate_equiv_bytes(ops, n, S))
    out = {"precision": precision, "ms_per_step": ms_step, "gbps": gb / (ms_step * 1e-3) / 1e9,
           "passes": st_plan["passes"], "rounds": st_plan["rounds"], "gates": st_plan["gates"],
           "pass_bytes": st_plan["pass_bytes"], "launches": int(launches),
           "specialised_passes": int(specialised), "warmup_s": round(warm_s, 2)}
    if per_pass:
        pm = np.concatenate(pass_ms)
        pt = np.concatenate(pass_ty)
        tile = pm[pt == 0]
        out["avg_tile_ms"] = float(tile.mean()) if tile.size else float(pm.mean())
        out["tile_bytes"] = 2.0 * S * 2 ** n
        out["tile_gbps"] = out["tile_bytes"] / (out["avg_tile_ms"] * 1e-3) / 1e9
    state.close()
    plan.close()
    return out


def plain_passes(n, ops, precision):
    """(forward passes, reverse-sweep passes) of the single-state adjoint
    plans (host planning only)."""
    import ctypes

    from pyquafu_gb300 import _native as nat
    from pyquafu_gb300 import ir

    lib = nat.load()
    arr, pool = ir.pack([o for o in ops if o.is_gate])
    prec = nat.PRECISIONS[precision]
    out = []
    for adjoint in (0, 1):
        h = ctypes.c_void_p()
        if adjoint:
            nat.check(lib.qfvm_plan_host_build_adjoint(n, prec, nat.vptr(arr), arr.size,
                                                       nat.dptr(pool.view(np.float64)), pool.size, ctypes.byref(h)))
        else:
            nat.check(lib.qfvm_plan_host_build(n, prec, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                                               pool.size, 0, 0, ctypes.byref(h)))
        counts = (ctypes.c_int64 * 4)()
        shape = (ctypes.c_int32 * 3)()
        nat.check(lib.qfvm_plan_host_counts(h, counts, shape))
        lib.qfvm_plan_destroy(h)
        out.append(int(counts[0]))
    return out[0], out[1]


def measure_adjoint(n=24, layers=20, ps_params=6, peak=FALLBACK_HBM, cpu=True, cpu_seconds=10.0, defer=None):
    """Adjoint gradients of a hardware-efficient ansatz (ry, rz on every qubit
    then a cx ladder, 2 * n * layers parameters; observable sum a_i Z_i Z_i+1 +
    sum b_i X_i): time per full gradient for each precision, its HBM rate
    (algorithmic bytes of the forward and reverse passes over the time), the
    same GPU's parameter-shift rate (timed on `ps_params` parameters, 2
    forward runs each, extrapolated), and the CPU baseline (the oracle's
    restatement of grad_adjoint, gradiant.py:144-173, its reverse sweep timed
    for `cpu_seconds` and extrapolated; appended to `defer` when given).
    Gradients are returned for the oracle comparison."""
    import torch

    from pyquafu_gb300 import batch as bmod
    from pyquafu_gb300 import gradients, workloads

    ops, _ = workloads.hea(n, layers, seed=0)
    terms = workloads.zz_x_hamiltonian(n, seed=0)
    nparam = 2 * n * layers
    out = {"workload": f"hea_{n}q_{layers}layers_{nparam}params_{len(terms)}terms"}
    grads = {}
    for prec in ("c128_ds", "c128", "c64"):
        gradients.adjoint(n, ops, terms, prec)  # warm-up (plans, allocation)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            e, g = gradients.adjoint(n, ops, terms, prec)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        fp, rp = plain_passes(n, ops, prec)
        nbytes = bmod.algorithmic_bytes(n, 1, fp, rp, S_OF[prec])
        out[prec] = {"s_per_gradient": round(dt, 4), "grads_per_s": round(nparam / dt, 1), "energy": e,
                     "passes": [fp, rp], "hbm_gbps": round(nbytes / dt / 1e9, 1),
                     "frac_hbm": round(nbytes / dt / 1e9 / peak, 4)}
        grads[prec] = g
    # parameter shift on the plain GPU path (complex128 FP64), a subset of parameters
    keep = set(range(ps_params))
    sub = [o if (o.slot in keep or o.slot < 0) else workloads.named(o.name, o.qubits, o.params) for o in ops]
    t0 = time.perf_counter()
    ps = gradients.param_shift(n, sub, terms, "c128")
    dt = time.perf_counter() - t0
    per_param = dt / max(1, len(keep))
    out["param_shift_c128"] = {"s_per_parameter": round(per_param, 4),
                               "s_per_gradient_extrapolated": round(per_param * nparam, 2),
                               "params_timed": len(keep),
                               "max_abs_diff_vs_adjoint": float(np.abs(ps[: len(keep)] - grads["c128"][: len(keep)]).max())}
    out["adjoint_speedup_vs_param_shift"] = {
        p: round(per_param * nparam / out[p]["s_per_gradient"], 1) for p in ("c128_ds", "c128", "c64")}
    def host_part():
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        fwd_s, lam_s, done, rev_s = oracle.grad_adjoint_timing(n, ops, [o.slot for o in ops], terms, cpu_seconds)
        total = fwd_s + lam_s + rev_s * len(ops) / max(done, 1)
        out["cpu_baseline"] = {"value": round(nparam / total, 2), "unit": "grads/s", "cores": os.cpu_count(),
                               "kind": "port", "s_per_gradient": round(total, 2),
                               "sample": f"oracle grad_adjoint: forward {fwd_s:.1f} s and lam {lam_s:.1f} s in full, "
                                         f"reverse sweep {done} of {len(ops)} gates in {rev_s:.1f} s, extrapolated"}

    if cpu:
        if defer is None:
            host_part()
        else:
            defer.append(host_part)
    return out, (ops, terms, grads)


def measure_uneven_batch(reps=5, check_items=8, cpu=True, cpu_seconds=8.0, tune=True, peak=FALLBACK_HBM):
    """2048 circuits of 10..18 qubits (ry encoding + 6 HEA layers), complex64
    with FP64 reductions: per-circuit <Z_0> and full gradient in one CUDA-graph
    launch.  Device time of the graph launch (uploads and downloads
    included), wall time through BatchSession.run, algorithmic bytes, and the
    complex64 error against the complex128 batched path on a subset."""
    from pyquafu_gb300 import batch as bmod
    from pyquafu_gb300 import workloads

    groups = workloads.uneven_batch()
    keys = sorted(groups)
    values = [groups[n][1] for n in keys]
    obs = [(1.0, "Z", [0])]
    tuned = {}
    if tune:
        from pyquafu_gb300 import autotune

        t0 = time.perf_counter()
        for n in keys:
            r = autotune.tune_batch_group(n, groups[n][0], groups[n][1], obs, "c64", reps=2)
            tuned[n] = [list(r["forward"]), list(r["reverse"])]
        tuned["seconds"] = round(time.perf_counter() - t0, 1)
    bs = bmod.BatchSession("c64", grads=True)
    nbytes = 0.0
    for n in keys:
        ops, vals = groups[n]
        bs.add_group(n, ops, obs, vals.shape[0], vals.shape[1])
        fp, rp = bmod.group_passes(n, ops, "c64")
        nbytes += bmod.algorithmic_bytes(n, vals.shape[0], fp, rp, 8)
    for _ in range(3):  # direct, capture + replay, replay
        bs.run(values, grads=True)
    dev = []
    t0 = time.perf_counter()
    for _ in range(reps):
        exps, grads, ms = bs.run(values, grads=True, timed=True)
        dev.append(ms)
    wall = (time.perf_counter() - t0) / reps
    info = bs.info()
    bs.close()
    ncirc = sum(v.shape[0] for v in values)
    ngrad = sum(v.size for v in values)
    dev_s = float(np.median(dev)) * 1e-3
    # complex64 error against the complex128 batched path (first items of every group)
    ref = bmod.BatchSession("c128", grads=True)
    sub = [v[:check_items] for v in values]
    for n, v in zip(keys, sub):
        ref.add_group(n, groups[n][0], obs, v.shape[0], v.shape[1])
    re_, rg_ = ref.run(sub, grads=True)
    ref.close()
    err_e = max(float(np.abs(e[:check_items] - r).max()) for e, r in zip(exps, re_))
    err_g = max(float(np.abs(g[:check_items] - r).max()) for g, r in zip(grads, rg_))
    out = {"workload": "uneven_batch_2048_circuits_10to18q_ry_encoding_6hea_layers_c64",
           "circuits": ncirc, "gradient_entries": ngrad, "groups": len(keys),
           "graph_launches_per_run": 1, "kernels_per_graph": int(info["kernels_per_run"][1]),
           "device_ms_per_run": round(dev_s * 1e3, 3), "wall_ms_per_run": round(wall * 1e3, 3),
           "circuits_per_s": round(ncirc / dev_s, 1), "grads_per_s": round(ngrad / dev_s, 1),
           "e2e_circuits_per_s": round(ncirc / wall, 1),
           "algorithmic_gb": round(nbytes / 1e9, 3), "achieved_gbps": round(nbytes / dev_s / 1e9, 1),
           "frac_hbm": round(nbytes / dev_s / 1e9 / peak, 4),
           "max_abs_err_vs_c128": {"expval": err_e, "grad": err_g, "items_checked": check_items * len(keys)},
           "autotuned_shapes": tuned}
    if cpu:
        out["cpu_baseline"] = cpu_batch_sample(groups, obs, cpu_seconds)
    return out


def cpu_batch_sample(groups, obs, seconds):
    """Reference algorithm on the host: the oracle port of grad_adjoint
    (gradiant.py:144-173) over the circuits of the smallest groups, until
    `seconds` have passed; circuits/s extrapolated by state size."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from pyquafu_gb300 import gradients

    oracle.build()
    done, cost_done, t0 = 0, 0.0, time.perf_counter()
    total_cost = sum(v.shape[0] * (2 ** n) for n, (_, v) in groups.items())
    for n in sorted(groups):
        ops, vals = groups[n]
        for v in vals:
            bound = gradients.bind(ops, v)
            oracle.grad_adjoint(n, bound, [o.slot for o in bound], obs)
            done += 1
            cost_done += 2 ** n
            if time.perf_counter() - t0 > seconds:
                break
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    rate = done / dt
    return {"value": round(rate * cost_done / done * sum(v.shape[0] for _, v in groups.values()) / total_cost, 2),
            "unit": "circuits/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{done} circuits (smallest qubit counts first) in {dt:.1f} s through the oracle's "
                      f"adjoint; rate scaled to the batch's size mix by 2^n"}


def measure_trajectories(n=18, shots=4096, cpu=True):
    """Per-shot trajectories: a random-layer circuit on n qubits with a
    measurement of two qubits, a reset and a classically controlled block in
    the middle, then a final measurement; every shot is one trajectory (the
    per-shot branch of simulate_circuit), all shots through one call."""
    from pyquafu_gb300 import ir, qfvm, workloads

    ops = workloads.random_layers(n, 6, seed=7)
    ops.append(ir.Op("measure", ir.OP_MEASURE, qbits=[0, 1], cbits=[0, 1]))
    ops.append(ir.Op("reset", ir.OP_RESET, qbits=[2]))
    ops.append(ir.Op("cif", ir.OP_CIF, cbits=[0, 1], condition=3,
                     body=[workloads.named("x", (2,)), workloads.named("h", (3,))]))
    ops += workloads.random_layers(n, 6, seed=8)
    ops.append(ir.Op("measure", ir.OP_MEASURE, qbits=list(range(4)), cbits=list(range(2, 6))))
    empty = np.zeros(0, dtype=np.complex128)
    qfvm._shots(n, 6, ops, empty, 64)  # warm-up
    t0 = time.perf_counter()
    out, _ = qfvm._shots(n, 6, ops, empty, shots)
    dt = time.perf_counter() - t0
    res = {"workload": f"random_layers_{n}q_12layers_midcircuit_measure_reset_cif", "shots": shots,
           "s_per_call": round(dt, 4), "shots_per_s": round(shots / dt, 1),
           "distinct_outcomes": int(len(set(out.tolist())))}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        k = 4
        uni = np.random.default_rng(0).random((k, ir.program_draws(ops)))
        t1 = time.perf_counter()
        oracle.simulate_shots(n, ops, 6, uni)
        cdt = (time.perf_counter() - t1) / k
        res["cpu_baseline"] = {"value": round(1.0 / cdt, 2), "unit": "shots/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"{k} shots through the oracle's per-shot restatement"}
    return res


def measure_noise(n=16, shots=2048, cpu=True):
    """Noisy trajectories (the NoiseSVSimulator workload): 8 random layers on
    n qubits with a depolarizing channel and an amplitude-damping channel on
    every qubit after every second layer; one sample and 3 Pauli terms per
    shot, all shots in one call."""
    from pyquafu_gb300 import ir, noise, workloads

    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]])
    Z = np.diag([1.0, -1.0]).astype(complex)
    p, g = 0.02, 0.05
    ops = []
    for layer in range(8):
        ops += workloads.random_layers(n, 1, seed=100 + layer)
        if layer % 2:
            for q in range(n):
                ops.append(ir.channel_op(ir.OP_UCHANNEL, q, [X, Y, Z, np.eye(2)], [p / 3, p / 3, p / 3, 1 - p]))
                ops.append(ir.channel_op(ir.OP_KRAUS, q, [np.array([[1, 0], [0, np.sqrt(1 - g)]]),
                                                          np.array([[0, np.sqrt(g)], [0, 0]])]))
    terms = [(1.0, "Z", [0]), (0.5, "ZZ", [0, 1]), (0.25, "X", [n - 1])]
    noise.simulate_noise(n, ops, 16, terms=terms)  # warm-up
    t0 = time.perf_counter()
    samples, expv = noise.simulate_noise(n, ops, shots, terms=terms)
    dt = time.perf_counter() - t0
    nch = sum(1 for o in ops if o.kind in (ir.OP_UCHANNEL, ir.OP_KRAUS))
    res = {"workload": f"random_layers_{n}q_8layers_{nch}channels_depolarizing_amplitude_damping", "shots": shots,
           "s_per_call": round(dt, 4), "shots_per_s": round(shots / dt, 1),
           "mean_expectations": [round(float(v), 6) for v in expv.mean(axis=0)]}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        k = 2
        uni = np.random.default_rng(0).random((k, ir.noise_draws(ops)))
        t1 = time.perf_counter()
        oracle.simulate_noise(n, ops, uni, terms=terms)
        cdt = (time.perf_counter() - t1) / k
        res["cpu_baseline"] = {"value": round(1.0 / cdt, 2), "unit": "shots/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"{k} shots through the oracle's noisy-trajectory restatement"}
    return res


def measure_qnn(steps=5, warmup=3, ps_forwards=20, tune=True, peak=FALLBACK_HBM, cpu=True, cpu_forwards=6):
    """QNN training step: 1024 samples x 16 qubits, 12 HEA layers (384 shared
    weights), MSE of <Z_0> against sign(w . x) labels; forward and adjoint
    backward through the torch binding (complex64, FP64 reductions), SGD
    update.  Compared with parameter shift on the plain GPU path:
    B * (1 + 2 * 384) single-circuit forward runs, timed on `ps_forwards`."""
    import torch

    from pyquafu_gb300 import batch as bmod
    from pyquafu_gb300 import gradients, workloads
    from pyquafu_gb300.engine import DeviceState
    from pyquafu_gb300.interface import QuantumLayer

    n, layers, B = 16, 12, 1024
    ops, w0, x, y = workloads.qnn_batch(batch=B, n=n, layers=layers)
    nw = 2 * n * layers
    tuned = None
    if tune:
        from pyquafu_gb300 import autotune

        v0 = np.concatenate([np.broadcast_to(w0, (B, nw)), x], axis=1)
        r = autotune.tune_batch_group(n, ops, v0, [(1.0, "Z", [0])], "c64", reps=2)
        tuned = {"forward": list(r["forward"]), "reverse": list(r["reverse"]), "forward_ms": r["forward_ms"],
                 "run_ms": r["run_ms"], "seconds": r["tuning_s"]}
    layer = QuantumLayer(n, ops, [(1.0, "Z", [0])], np.arange(nw), nw + np.arange(n), init=w0, precision="c64")
    opt = torch.optim.SGD(layer.parameters(), lr=0.05)
    xt, yt = torch.tensor(x), torch.tensor(y)

    def step():
        opt.zero_grad()
        out = layer(xt)
        loss = torch.mean((out[:, 0] - yt) ** 2)
        loss.backward()
        opt.step()
        return float(loss.detach())

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    losses = [step() for _ in range(steps)]
    dt = (time.perf_counter() - t0) / steps
    # device time of one forward + adjoint run of the batch
    runner = layer.runner(B)
    vals = np.concatenate([np.broadcast_to(layer.weight.detach().numpy(), (B, nw)), x], axis=1)
    dev = []
    for _ in range(3):
        dev.append(runner.session.run([vals], grads=True, timed=True)[2])
    dev_s = float(np.median(dev)) * 1e-3
    fp, rp = bmod.group_passes(n, ops, "c64")
    nbytes = bmod.algorithmic_bytes(n, B, fp, rp, 8)
    # parameter shift on the plain path: one forward per evaluation
    st = DeviceState(n, "c64")
    terms = [(1.0, "Z", [0])]
    bound = gradients.bind(ops, vals[0])
    gradients.energy(n, bound, terms, "c64", st)
    t1 = time.perf_counter()
    for _ in range(ps_forwards):
        gradients.energy(n, bound, terms, "c64", st)
    fwd_s = (time.perf_counter() - t1) / ps_forwards
    st.close()
    ps_step = B * (1 + 2 * nw) * fwd_s
    # the same parameter-shift algorithm with every shifted evaluation an
    # item of a batched run (4 samples timed, extrapolated to the batch)
    sub = 4
    gradients.jacobian_param_shift(n, ops, [(1.0, "Z", [0])], vals[:1], "c64")  # warm-up
    t2 = time.perf_counter()
    gradients.jacobian_param_shift(n, ops, [(1.0, "Z", [0])], vals[:sub], "c64")
    psb = (time.perf_counter() - t2) / sub * B
    cpu_base = None
    if cpu:
        # the reference's ExecuteCircuits step on the host: B forward
        # evaluations, then B * 2 * 384 shifted evaluations for the
        # parameter-shift Jacobian (torch.py:65-89, vjp.py:60-103), each a
        # simulation of the circuit and <Z_0> through the oracle
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        t3 = time.perf_counter()
        for k in range(cpu_forwards):
            b_ops = gradients.bind(ops, vals[k])
            oracle.expect_pauli(oracle.simulate(n, b_ops), "Z", [0])
        cfw = (time.perf_counter() - t3) / cpu_forwards
        cstep = B * (1 + 2 * nw) * cfw
        cpu_base = {"value": round(1.0 / cstep, 9), "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                    "s_per_step": round(cstep, 1),
                    "sample": f"{cpu_forwards} oracle forward evaluations ({cfw * 1e3:.1f} ms each) extrapolated to "
                              f"{B} x (1 + 2 x {nw}) evaluations per step"}
    return {"workload": "qnn_1024x16q_12hea_layers_384_weights_mse_z0_c64", "cpu_baseline": cpu_base,
            "frac_hbm": round(nbytes / dev_s / 1e9 / peak, 4),
            "param_shift_batched": {"samples_timed": sub, "evaluations_per_sample": 1 + 2 * nw,
                                    "s_per_step_extrapolated": round(psb, 2),
                                    "adjoint_speedup": round(psb / dt, 1)},
            "s_per_step": round(dt, 5), "steps_per_s": round(1 / dt, 2),
            "device_ms_forward_adjoint": round(dev_s * 1e3, 3),
            "algorithmic_gb": round(nbytes / 1e9, 3), "achieved_gbps": round(nbytes / dev_s / 1e9, 1),
            "passes": {"forward": fp, "reverse": rp}, "loss_first_last": [losses[0], losses[-1]],
            "param_shift_plain_path": {"s_per_forward": round(fwd_s, 6), "forwards_per_step": B * (1 + 2 * nw),
                                       "s_per_step_extrapolated": round(ps_step, 1)},
            "speedup_vs_param_shift": round(ps_step / dt, 1), "autotuned": tuned}


def measure_c1(steps=20, shots=4096, cpu=True, peak=FALLBACK_HBM, defer=None):
    """The 20-qubit random circuit (depth 20, seed 0, complex128) with 4096
    shots: gate time on the device (the 16 MiB state stays in L2 between
    steps, so its GB/s are L2-resident figures), sampling time (one call:
    uniforms up, block sums, block prefix, per-shot locate, exact fallback,
    indices down), shots the exact scan resolved, and the oracle's gate and
    sequential-scan times on the host cores (statevector.hpp:1380-1412 is
    serial).  Errors: final state against the oracle per amplitude, sampled
    indices against the oracle's scan with the same seeded uniforms.  With
    `defer` (a list) the host part is appended to it instead of run."""
    import torch

    from pyquafu_gb300 import engine, workloads

    n = 20
    ops = workloads.random_layers(n, 20, seed=0)
    out = {"workload": f"random_layers_{n}q_c128_depth20_{shots}shots", "gates": len(ops)}
    u = np.random.Generator(np.random.MT19937(0)).random(shots)
    states = {}
    for prec in ("c128_ds", "c128"):
        plan = engine.Plan(n, ops, prec)
        st = engine.DeviceState(n, prec).set_zero()
        for _ in range(3):
            st.set_zero()
            plan.run(st)
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            st.set_zero()
            p_ms, _ = plan.run_timed(st)
            ms.append(float(np.sum(p_ms)))
        st.set_zero()
        plan.run(st)
        torch.cuda.synchronize()
        gms = float(np.median(ms))
        gb = sum(gate_equiv_bytes(ops, n, 16))
        row = {"gates_ms": round(gms, 3), "gbps_gate_equiv_l2_resident": round(gb / (gms * 1e-3) / 1e9, 1),
               "passes": plan.stats()["passes"]}
        if prec == "c128_ds":
            st.sample(u)  # warm-up
            t0 = time.perf_counter()
            reps = 5
            for _ in range(reps):
                idx = st.sample(u)
            row["sample_ms"] = round((time.perf_counter() - t0) / reps * 1e3, 3)
            row["sequential_blocks"] = st.sequential_blocks()
            out["indices"] = idx
        states[prec] = st.download()
        st.close()
        plan.close()
        out[prec] = row
    indices = out.pop("indices")

    def host_part():
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        t0 = time.perf_counter()
        ref = oracle.simulate(n, ops)
        t1 = time.perf_counter()
        ref_idx = oracle.sample_indices(ref, u)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"gates_s": round(t1 - t0, 3), "scan_s": round(t2 - t1, 3), "kind": "port",
                               "cores": os.cpu_count(), "cpu": cpu_info(),
                               "sample": "the full circuit and all 4096 shots (sequential scan, one core)"}
        for prec in ("c128_ds", "c128"):
            out[prec]["max_abs_err_vs_oracle"] = max_abs_diff(states[prec], ref)
        out["sample_mismatches_vs_oracle"] = int(np.sum(indices != ref_idx))

    if cpu:
        if defer is None:
            host_part()
        else:
            defer.append(host_part)
    return out


SHOT_SEED = 0
SHOTS = 4096


class OracleRun:
    """The oracle's full run of the benchmark circuit on the host cores, in a
    child process forked before the first GPU call, so it runs while the
    device-timed rows do (rows whose figures include host time wait for it).
    The final state lands in an anonymous shared mapping; the child also
    computes <Z0 Z1> and the indices of the 4096 seeded shots (the oracle's
    single-walk scan, equal to its per-shot scan).  The fork also comes
    before this process's first oracle call: the oracle's OpenMP runtime
    does not carry its thread pool across a fork, and a child forked after
    a parallel region waits in its first one."""

    def __init__(self, n, ops):
        import mmap

        self.n = n
        self.u = np.random.Generator(np.random.MT19937(SHOT_SEED)).random(SHOTS)
        self._map = mmap.mmap(-1, (16 << n) + 8 * (4 + SHOTS))
        self.pid = os.fork()
        if self.pid == 0:  # child: no GPU, no torch
            code = 1
            try:
                sys.path.insert(0, os.path.join(ROOT, "oracle"))
                import oracle

                oracle.build()
                psi = self._state()
                hdr = self._header()
                t0 = time.perf_counter()
                psi[:] = 0
                psi[0] = 1.0
                for op in ops:
                    oracle.apply_op(psi, op)
                hdr[0] = time.perf_counter() - t0
                hdr[1] = oracle.expect_pauli(psi, "ZZ", [0, 1])
                t1 = time.perf_counter()
                self._indices()[:] = oracle.sample_indices_sorted(psi, self.u)
                hdr[2] = time.perf_counter() - t1
                hdr[3] = 1.0
                code = 0
            except BaseException as e:  # reported by the parent as a failed check
                print(f"[bench] oracle run failed: {e!r}", file=sys.stderr, flush=True)
            finally:
                os._exit(code)
        import atexit

        atexit.register(self.abandon)  # registered in the parent only, after the fork

    def abandon(self):
        """Ends the child (its exact pid) when the bench stops without
        waiting for it, e.g. after an exception in the GPU rows."""
        if self.pid:
            import signal

            try:
                os.kill(self.pid, signal.SIGKILL)
                os.waitpid(self.pid, 0)
            except OSError:
                pass
            self.pid = 0

    def _state(self):
        return np.frombuffer(self._map, dtype=np.complex128, count=1 << self.n)

    def _header(self):
        return np.frombuffer(self._map, dtype=np.float64, count=4, offset=16 << self.n)

    def _indices(self):
        return np.frombuffer(self._map, dtype=np.uint64, count=SHOTS, offset=(16 << self.n) + 32)

    def result(self):
        """Waits for the child; (state, <Z0Z1>, shot indices, seconds of the
        circuit, seconds of the scan), or None when it failed."""
        if self.pid:
            _, status = os.waitpid(self.pid, 0)
            self.pid = 0
            self.status = status
        hdr = self._header()
        if hdr[3] != 1.0:
            return None
        return self._state(), float(hdr[1]), self._indices(), float(hdr[0]), float(hdr[2])


def oracle_check_c2(n, ops, precisions, run):
    """Final state of every arithmetic against the oracle's full run (`run`,
    an OracleRun), per amplitude, and <Z0 Z1>; the first arithmetic's 4096
    shots against the oracle's scan with the same seeded uniforms."""
    import torch

    from pyquafu_gb300 import engine

    res = run.result()
    if res is None:
        return {"error": "the oracle run failed (see stderr)"}
    ref, zz_ref, ref_idx, oracle_s, scan_s = res
    out = {"oracle_full_circuit_s": round(oracle_s, 1), "oracle_cores": os.cpu_count()}
    buf = np.empty(1 << n, dtype=np.complex128)
    for prec in precisions:
        plan = engine.Plan(n, ops, prec)
        st = engine.DeviceState(n, prec).set_zero()
        plan.run(st)
        torch.cuda.synchronize()
        zz = float(st.expect([("ZZ", [0, 1])])[0])
        if prec == precisions[0]:
            # 4096 shots on the final state, exact against the oracle's scan
            st.sample(run.u)
            t0 = time.perf_counter()
            idx = st.sample(run.u)
            sample_ms = (time.perf_counter() - t0) * 1e3
            out["sampling_4096_shots"] = {"gpu_ms": round(sample_ms, 2), "sequential_blocks": st.sequential_blocks(),
                                          "oracle_scan_s": round(scan_s, 2),
                                          "oracle_scan": "one walk of the FP64 running sum, shots by ascending "
                                                         "uniform (equal to the per-shot scan)",
                                          "mismatches_vs_oracle": int(np.sum(idx != ref_idx))}
        st.download(buf)
        st.close()
        plan.close()
        out[prec] = {"max_abs_err": max_abs_diff(buf, ref), "zz_abs_err": abs(zz - zz_ref)}
    return out


class Sections:
    """Wall time of each part of the run, on stderr as it goes."""

    def __init__(self):
        self.t = {}

    def __call__(self, name, fn, *a, **k):
        t0 = time.perf_counter()
        r = fn(*a, **k)
        self.t[name] = round(time.perf_counter() - t0, 1)
        print(f"[bench] {name}: {self.t[name]} s", file=sys.stderr, flush=True)
        return r


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: replicas run independent batches, so the
    job's time is the maximum over ranks (all-reduce MAX; no data-path
    collective exists)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def autotune_all(args, n, ops):
    """Pick the fused-pass shapes for every workload of this run with the
    project autotuner (pyquafu_gb300.autotune); tuning time is reported and
    is outside every timed region."""
    from pyquafu_gb300 import autotune, workloads

    t0 = time.perf_counter()
    out = {}
    proxy = min(n, 26)
    pops = workload(proxy)
    for prec in [args.precision] + [v for v in args.variants.split(",") if v and v != args.precision]:
        r = autotune.tune_plan(proxy, pops, prec, reps=2, apply_to=[n])
        out[f"plan_{prec}"] = {"tuned_on_qubits": proxy, "shape": r["shape"], "times_ms": r["times_ms"]}
    if not args.skip_adjoint:
        aops, _ = workloads.hea(args.adjoint_qubits, 20, seed=0)
        terms = workloads.zz_x_hamiltonian(args.adjoint_qubits, seed=0)
        for prec in ("c128", "c128_ds", "c64"):
            r = autotune.tune_adjoint(args.adjoint_qubits, aops, terms, prec, reps=1)
            out[f"adjoint_{prec}"] = {"shape": r["shape"], "times_ms": r["times_ms"]}
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def run_gpu(args):
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    n = N_QUBITS
    ops = workload()
    # the oracle's full run starts first, in a child forked before any GPU call
    oracle_run = OracleRun(n, ops) if rank == 0 and not args.skip_oracle_check else None
    sec = Sections()

    import torch

    from pyquafu_gb300 import _native as nat
    from pyquafu_gb300 import qfvm, workloads
    from pyquafu_gb300.builder import build

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    build()
    nat.load()
    peak, peak_kind = hbm_peak()
    cpu_here = rank == 0 and not args.skip_cpu

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    tuning = None if args.no_autotune else sec("autotune", autotune_all, args, n, ops)
    barrier()
    clocks = ClockSampler()
    clocks.start()
    main = sec("headline", measure, args.precision, ops, n, args.steps, args.warmup)
    clk = clocks.stop()
    barrier()
    total_ms = max_over_ranks(main["ms_per_step"] * args.steps, world, "cuda")
    ms_step = total_ms / args.steps
    S = S_OF[args.precision]
    gb = sum(gate_equiv_bytes(ops, n, S))
    value = world * gb / (ms_step * 1e-3) / 1e9
    achieved = main["tile_gbps"]

    variants = {}
    for v in [x for x in args.variants.split(",") if x and x != args.precision]:
        r = sec(f"variant {v}", measure, v, ops, n, min(args.steps, 3), max(1, min(args.warmup, 3)))
        variants[v] = {"value": round(r["gbps"], 2), "unit": "GB/s", "ms_per_step": round(r["ms_per_step"], 3),
                       "passes": r["passes"], "tile_kernel": kernel_name(v, n, r["specialised_passes"] > 0),
                       "specialised_passes": r["specialised_passes"], "tile_pass_gbps": round(r["tile_gbps"], 1),
                       "tile_pass_frac_hbm": round(r["tile_gbps"] / peak, 4),
                       "hbm_gbps": round(r["pass_bytes"] / (r["ms_per_step"] * 1e-3) / 1e9, 1)}

    # device-timed rows whose host parts wait for the oracle run
    deferred = []
    c1 = None if args.skip_c1 else sec("C1", measure_c1, cpu=cpu_here, peak=peak, defer=deferred)
    adj = adj_data = None
    if not args.skip_adjoint:
        adj, adj_data = sec("C3 adjoint", measure_adjoint, args.adjoint_qubits, peak=peak, cpu=cpu_here,
                            defer=deferred)
    if oracle_run is not None:
        sec("oracle run (wait)", oracle_run.result)

    # --- end to end through the reference-shaped API (host buffers) ---
    e2e = None
    if not args.skip_e2e:
        qfvm.set_arithmetic("ds" if args.precision == "c128_ds" else "fp64")
        host = torch.empty(2 * 2 ** n, dtype=torch.float64, pin_memory=True)
        psi = host.numpy().view(np.complex128)
        psi[:] = 0
        psi[0] = 1.0
        circuit = workloads.as_protocol(n, ops)
        qfvm.simulate_circuit(circuit, psi, 0)
        torch.cuda.synchronize()
        t_e2e = time.perf_counter()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            qfvm.simulate_circuit(circuit, psi, 0)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
        gb128 = sum(gate_equiv_bytes(ops, n, 16))
        e2e = {"value": round(world * gb128 / e2e_s / 1e9, 2), "unit": "GB/s",
               "h2d_bytes_per_step": int(16 * 2 ** n), "d2h_bytes_per_step": int(16 * 2 ** n),
               "ms_per_step": round(e2e_s * 1e3, 2), "arithmetic": qfvm.get_arithmetic(),
               "api": "pyquafu_gb300.qfvm.simulate_circuit(circuit, pinned complex128 state, shots=0)"}
        del psi, host
        qfvm.set_arithmetic("ds")
        print(f"[bench] e2e: {time.perf_counter() - t_e2e:.1f} s", file=sys.stderr, flush=True)

    batched = None
    if not args.skip_batch:
        batched = {}
        if not args.skip_uneven:
            batched["uneven_2048"] = sec("C4 batch", measure_uneven_batch, cpu=cpu_here, tune=not args.no_autotune,
                                         peak=peak)
        batched["qnn_training_step"] = sec("C5 qnn", measure_qnn, tune=not args.no_autotune, peak=peak, cpu=cpu_here)
        if not args.skip_trajectories:
            batched["trajectories"] = sec("trajectories", measure_trajectories, cpu=cpu_here)
            batched["noise"] = sec("noise", measure_noise, cpu=cpu_here)
    for i, part in enumerate(deferred):
        sec(f"host part {i}", part)

    cpu = None
    if cpu_here:
        cgbps, gates_done, cdt = sec("cpu baseline", cpu_sample, ops, n, seconds=args.cpu_seconds)
        info = cpu_info()
        cpu = {"value": round(cgbps, 3), "unit": "GB/s", "cores": info["cores"], "kind": "port",
               "sample": f"{gates_done} gates of the circuit in strided order on the {n}-qubit complex128 state "
                         f"({cdt:.1f} s, OpenMP over all cores)", "cpu": info}

    # --- the error of every result against the oracle (after all timing) ---
    check = None
    if oracle_run is not None:
        precs = [args.precision] + [v for v in args.variants.split(",") if v and v != args.precision]
        check = sec("oracle check", oracle_check_c2, n, ops, precs, oracle_run)
        if adj_data is not None:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle

            aops, aterms, grads = adj_data
            t0 = time.perf_counter()
            gref = oracle.grad_adjoint(args.adjoint_qubits, aops, [o.slot for o in aops], aterms)
            adj["oracle_s"] = round(time.perf_counter() - t0, 1)
            for prec, g in grads.items():
                adj[prec]["max_abs_err_vs_oracle"] = float(np.abs(g - gref).max())

    if rank == 0:
        err = (check or {}).get(args.precision, {})
        line = {
            "metric": "statevector_gbps", "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"c128": "f64", "c128_ds": "f32x2", "c64": "f32"}[args.precision],
            "data": "synthetic",
            "config": config_of(n, ops),
            "engine": {"precision": args.precision, "storage": "c64" if args.precision == "c64" else "c128",
                       "passes": main["passes"], "rounds": main["rounds"],
                       "parallelism": "replicas" if world > 1 else "single"},
            "max_abs_err_vs_oracle": err.get("max_abs_err"),
            "roofline": {"bound": "hbm", "kernel": kernel_name(args.precision, n, main["specialised_passes"] > 0),
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "traffic": (round(TRAFFIC_PER_AMP[args.precision] * 2 ** n)
                                     if args.precision in TRAFFIC_PER_AMP else None),
                         "traffic_source": ("ncu dram bytes of a 26-qubit launch, scaled by 2^(n-26)"
                                            if args.precision in TRAFFIC_PER_AMP else None),
                         "bytes_per_launch": main["tile_bytes"], "avg_launch_ms": round(main["avg_tile_ms"], 3)},
            "hbm_gbps": round(main["pass_bytes"] / (ms_step * 1e-3) / 1e9, 1),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(main["launches"]),
            "specialised": {"passes": main["specialised_passes"], "of": main["passes"],
                            "first_runs_s": main["warmup_s"]},
            "autotune": tuning,
            "variants": variants,
            "oracle_check": check,
            "c1_sampling": c1,
            "adjoint": adj,
            "batched": batched,
        }
        line["rows"] = summary_rows(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def _r(x, nd=4):
    return None if x is None else (round(x, nd) if isinstance(x, float) else x)


def summary_rows(line):
    """Compact per-configuration figures, printed last on the line."""
    rows = {}
    chk = line.get("oracle_check") or {}
    c2 = {line["engine"]["precision"]: {"ms": line["ms_per_step"], "frac": line["roofline"]["frac"],
                                        "err": chk.get(line["engine"]["precision"], {}).get("max_abs_err")}}
    for v, r in (line.get("variants") or {}).items():
        c2[v] = {"ms": r["ms_per_step"], "frac": r["tile_pass_frac_hbm"], "err": chk.get(v, {}).get("max_abs_err")}
    if "sampling_4096_shots" in chk:
        c2["sampling_4096_shots"] = chk["sampling_4096_shots"]
    rows["C2_30q"] = c2
    c1 = line.get("c1_sampling")
    if c1:
        cb = c1.get("cpu_baseline") or {}
        rows["C1_20q_4096shots"] = {"gates_ms": c1["c128_ds"]["gates_ms"], "sample_ms": c1["c128_ds"]["sample_ms"],
                                    "sequential_blocks": c1["c128_ds"]["sequential_blocks"],
                                    "err": c1["c128_ds"].get("max_abs_err_vs_oracle"),
                                    "sample_mismatches": c1.get("sample_mismatches_vs_oracle"),
                                    "cpu_gates_s": cb.get("gates_s"), "cpu_scan_s": cb.get("scan_s")}
    a = line.get("adjoint")
    if a:
        rows["C3_24q_adjoint"] = {p: {"s": a[p]["s_per_gradient"], "frac": a[p]["frac_hbm"],
                                      "err": a[p].get("max_abs_err_vs_oracle")} for p in ("c128_ds", "c128", "c64")}
        rows["C3_24q_adjoint"]["vs_param_shift"] = a["adjoint_speedup_vs_param_shift"]
        rows["C3_24q_adjoint"]["cpu_s"] = (a.get("cpu_baseline") or {}).get("s_per_gradient")
    b = line.get("batched") or {}
    if "uneven_2048" in b:
        u = b["uneven_2048"]
        rows["C4_2048_circuits"] = {"circuits_per_s": u["circuits_per_s"], "frac": u["frac_hbm"],
                                    "err_vs_c128": u["max_abs_err_vs_c128"]["grad"],
                                    "cpu_circuits_per_s": (u.get("cpu_baseline") or {}).get("value")}
    if "qnn_training_step" in b:
        q = b["qnn_training_step"]
        rows["C5_qnn_step"] = {"steps_per_s": q["steps_per_s"], "frac": q["frac_hbm"],
                               "vs_param_shift": q["speedup_vs_param_shift"],
                               "cpu_s_per_step": (q.get("cpu_baseline") or {}).get("s_per_step")}
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default=DEFAULT_PRECISION, choices=["c128", "c128_ds", "c64"])
    ap.add_argument("--variants", default="c128,c64")
    ap.add_argument("--skip-c1", action="store_true")
    ap.add_argument("--skip-uneven", action="store_true")
    ap.add_argument("--skip-trajectories", action="store_true")
    ap.add_argument("--skip-oracle-check", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-variants", action="store_true")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--adjoint-qubits", type=int, default=24)
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    if args.skip_variants:
        args.variants = ""
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
