"""Autotuner for the fused-pass shapes.

A fused pass is compiled for a few shapes (tile qubits T, register qubits R,
tile buffers, resident CTAs per SM); which one is fastest depends on the
precision, the qubit count and the gate mix.  The tuner times every compiled
shape on the caller's own workload with CUDA events, records the winner in
the engine's process-wide shape table (``qfvm_set_tuned_shape``: every later
plan or batch group of that precision and qubit count uses it) and keeps it
in a JSON cache keyed by device name, precision, pass kind and qubit count.

Pass kinds: 0 = one-state passes (simulation, forward of a batch), 1 =
two-state passes of the adjoint reverse sweep.

Cache file: ``$QFVM_AUTOTUNE_CACHE`` or ``~/.cache/pyquafu_gb300/autotune.json``.
"""

from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import _native as nat
from .engine import DeviceState, Plan, _precision

KINDS = (0, 1)


def cache_path() -> str:
    return os.environ.get("QFVM_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "pyquafu_gb300", "autotune.json")


def device_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:  # no torch / no device: one shared key
        return "unknown"


def candidates(precision, kind: int) -> list[tuple[int, int]]:
    """Compiled (T, R) shapes of a pass kind."""
    lib = nat.load()
    p = _precision(precision)
    return [(t, r) for t in range(6, 16) for r in range(2, 7)
            if r < t and lib.qfvm_shape_supported(p, kind, t, r)]


def current(precision, kind: int, n: int) -> tuple[int, int]:
    lib = nat.load()
    t, r = ctypes.c_int32(), ctypes.c_int32()
    nat.check(lib.qfvm_get_shape(_precision(precision), kind, n, ctypes.byref(t), ctypes.byref(r)), "get shape")
    return t.value, r.value


def set_shape(precision, kind: int, n: int, shape) -> None:
    lib = nat.load()
    t, r = shape if shape else (0, 0)
    nat.check(lib.qfvm_set_tuned_shape(_precision(precision), kind, int(n), int(t), int(r)), "set shape")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(precision, kind, n, shape, ms) -> None:
    data = _load()
    ent = data.setdefault(device_name(), {}).setdefault(str(precision), {}).setdefault(str(kind), {})
    ent[str(n)] = {"shape": list(shape), "ms": ms}
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home still gets the in-process table


def apply_cached() -> int:
    """Load this device's cached shapes into the engine; returns how many."""
    count = 0
    for prec, kinds in _load().get(device_name(), {}).items():
        for kind, ns in kinds.items():
            for n, ent in ns.items():
                try:
                    set_shape(prec, int(kind), int(n), tuple(ent["shape"]))
                    count += 1
                except nat.QfvmError:
                    pass  # a shape the library no longer compiles
    return count


def _sync():
    try:
        import torch

        torch.cuda.synchronize()
    except Exception:
        pass


def tune_plan(n: int, ops, precision="c128", reps: int = 2, apply_to=None) -> dict:
    """Time the one-state plan of ``ops`` under every compiled shape (pass
    kind 0) and record the fastest for ``n`` (and for every qubit count in
    ``apply_to``: a smaller proxy circuit can tune a larger one)."""
    st = DeviceState(n, precision)
    times = {}
    for shape in candidates(precision, 0):
        if shape[0] > n:
            continue
        plan = Plan(n, ops, precision, *shape)
        st.set_zero()
        plan.run_timed(st)  # warm-up
        ms = []
        for _ in range(reps):
            st.set_zero()
            ms.append(float(np.sum(plan.run_timed(st)[0])))
        plan.close()
        times[shape] = min(ms)
    st.close()
    if not times:
        return {"n": n, "shape": None, "times_ms": {}}
    best = min(times, key=times.get)
    for m in [n] + list(apply_to or []):
        set_shape(precision, 0, m, best)
        _store(precision, 0, m, best, times[best])
    return {"n": n, "shape": best, "times_ms": {f"{t},{r}": round(v, 3) for (t, r), v in times.items()}}


def tune_batch_group(n: int, ops, values, observables, precision="c64", reps: int = 3) -> dict:
    """Tune the forward shape (mode 0 runs) and then the reverse-sweep shape
    (mode 1 runs) for one batch group of n qubits with the given per-item
    values; records both for n."""
    from .batch import BatchSession

    values = np.asarray(values, dtype=np.float64)
    items, slots = values.shape

    def timed(fwd, rev, grads):
        bs = BatchSession(precision, grads=grads, tile=fwd, adjoint_tile=rev)
        bs.add_group(n, ops, observables, items, slots)
        for _ in range(2):  # direct run, then graph capture
            bs.run([values], grads=grads)
        ms = min(bs.run([values], grads=grads, timed=True)[-1] for _ in range(reps))
        bs.close()
        return ms

    t0 = time.perf_counter()
    fwd_times = {s: timed(s, None, False) for s in candidates(precision, 0)}
    best_fwd = min(fwd_times, key=fwd_times.get)
    rev_times = {s: timed(best_fwd, s, True) for s in candidates(precision, 1)}
    best_rev = min(rev_times, key=rev_times.get)
    set_shape(precision, 0, n, best_fwd)
    set_shape(precision, 1, n, best_rev)
    _store(precision, 0, n, best_fwd, fwd_times[best_fwd])
    _store(precision, 1, n, best_rev, rev_times[best_rev])
    return {"n": n, "forward": best_fwd, "reverse": best_rev,
            "forward_ms": {f"{t},{r}": round(v, 3) for (t, r), v in fwd_times.items()},
            "run_ms": {f"{t},{r}": round(v, 3) for (t, r), v in rev_times.items()},
            "tuning_s": round(time.perf_counter() - t0, 2)}


def tune_adjoint(n: int, ops, terms, precision="c128", reps: int = 2) -> dict:
    """Time the single-state adjoint gradient (forward, lam = H psi, reverse
    sweep) under every compiled reverse-sweep shape (pass kind 1) and record
    the fastest for n."""
    from . import gradients

    times = {}
    keep = current(precision, 1, n)
    for shape in candidates(precision, 1):
        set_shape(precision, 1, n, shape)
        gradients.adjoint(n, ops, terms, precision)  # warm-up
        ms = []
        for _ in range(reps):
            _sync()
            t0 = time.perf_counter()
            gradients.adjoint(n, ops, terms, precision)
            _sync()
            ms.append((time.perf_counter() - t0) * 1e3)
        times[shape] = min(ms)
    if not times:
        set_shape(precision, 1, n, keep)
        return {"n": n, "shape": None, "times_ms": {}}
    best = min(times, key=times.get)
    set_shape(precision, 1, n, best)
    _store(precision, 1, n, best, times[best])
    return {"n": n, "shape": best, "times_ms": {f"{t},{r}": round(v, 3) for (t, r), v in times.items()}}
