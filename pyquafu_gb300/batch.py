"""Batched runs on the GB300 engine (the ``qfvm_batch_*`` C ABI).

The reference evaluates a batch one sample at a time from Python
(quafu/algorithms/interface/torch.py:76-78 calls ``run_circ`` per sample,
quafu/algorithms/gradients/vjp.py:93-103 runs ``ParamShift`` per sample and
observable).  Here a batch is one device run: circuits that share a gate
structure form a group whose states sit back to back in HBM, every fused pass
covers all items of the group, per-item angles are bound on the device, and
groups of different qubit counts run side by side.  After the first run of
a mode the whole run (uploads, every kernel of every group, downloads) is
replayed as one CUDA graph launch.

A group is given by its gate list (``ir.Op`` records; a gate with ``slot >= 0``
takes its angle from the item's value vector), its observables (each a list of
``(coeff, paulistr, pos)`` terms), the number of items and the number of slots.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from . import ir
from .engine import _precision, pack_terms

GRADS = 1
NO_GRAPH = 2


def _observables(observables):
    """Normalise to a list of observables (each a list of terms)."""
    if not observables:
        raise ValueError("a group needs at least one observable")
    first = observables[0]
    if isinstance(first, tuple) and len(first) == 3 and isinstance(first[1], str):
        return [list(observables)]  # a single observable given as its term list
    return [list(o) for o in observables]


class BatchSession:
    """Owns a ``qfvm_batch``: groups of same-structure circuits evaluated in
    one device run.  ``grads=True`` prepares adjoint-gradient runs."""

    def __init__(self, precision="c64", grads: bool = True, graph: bool = True, tile=None, adjoint_tile=None):
        """``tile`` / ``adjoint_tile``: (tile qubits, register qubits) of the
        forward / reverse-sweep passes (None: the engine's defaults)."""
        lib = nat.load()
        self._lib = lib
        self.precision = precision
        self.grads = bool(grads)
        flags = (GRADS if grads else 0) | (0 if graph else NO_GRAPH)
        t, r = tile if tile else (0, 0)
        at, ar = adjoint_tile if adjoint_tile else (0, 0)
        shapes = np.array([t, r, at, ar], dtype=np.int32)
        h = ctypes.c_void_p()
        nat.check(lib.qfvm_batch_create(_precision(precision), flags, nat.i32ptr(shapes), ctypes.byref(h)),
                  "batch create")
        self._h = h
        self.groups = []  # (n, items, slots, nobs)

    def add_group(self, n: int, ops, observables, items: int, slots: int | None = None) -> int:
        gates = [o for o in ops if o.is_gate]
        if len(gates) != len(ops):
            raise ValueError("batched groups take gates only (no measure/reset/cif)")
        if slots is None:
            slots = max([o.slot for o in gates] + [-1]) + 1
        obs = _observables(observables)
        terms, owner = [], []
        for k, o in enumerate(obs):
            for t in o:
                terms.append(t)
                owner.append(k)
        x, z, y = pack_terms([(p, pos) for _, p, pos in terms])
        c = np.array([float(np.real(t[0])) for t in terms], dtype=np.float64)
        oi = np.array(owner, dtype=np.int32)
        arr, pool = ir.pack(gates)
        rc = self._lib.qfvm_batch_add_group(self._h, int(n), nat.vptr(arr), arr.size,
                                            nat.dptr(pool.view(np.float64)), pool.size, nat.u64ptr(x),
                                            nat.u64ptr(z), nat.i32ptr(y), nat.dptr(c), nat.i32ptr(oi), c.size,
                                            len(obs), int(items), int(slots))
        nat.check(rc, "batch add_group")
        self.groups.append((int(n), int(items), int(slots), len(obs)))
        return len(self.groups) - 1

    # ------------------------------------------------------------------ runs

    def _pack_values(self, values):
        if len(values) != len(self.groups):
            raise ValueError(f"expected values for {len(self.groups)} groups, got {len(values)}")
        parts = []
        for (n, items, slots, _), v in zip(self.groups, values):
            v = np.asarray(v, dtype=np.float64)
            if v.shape != (items, slots):
                raise ValueError(f"group values must have shape {(items, slots)}, got {v.shape}")
            parts.append(v.reshape(-1))
        return np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(0))

    def _pack_weights(self, weights):
        if weights is None:
            return None
        parts = []
        for (n, items, slots, nobs), w in zip(self.groups, weights):
            w = np.asarray(w, dtype=np.float64)
            if w.shape != (items, nobs):
                raise ValueError(f"group weights must have shape {(items, nobs)}, got {w.shape}")
            parts.append(w.reshape(-1))
        return np.ascontiguousarray(np.concatenate(parts))

    def run(self, values, grads: bool = False, weights=None, timed: bool = False):
        """values: per group an (items, slots) array.  Returns per group the
        (items, nobs) expectation values and, with ``grads``, the (items,
        slots) gradients of sum_o weights[item, o] <O_o> (weights default 1).
        With ``timed`` the device time of the run (ms) is returned last."""
        if grads and not self.grads:
            raise ValueError("this session was created without gradient support")
        vals = self._pack_values(values)
        w = self._pack_weights(weights) if grads else None
        nexp = sum(i * o for _, i, _, o in self.groups)
        ngrad = sum(i * s for _, i, s, _ in self.groups) if self.grads else 0
        ev = np.zeros(max(nexp, 1))
        gr = np.zeros(max(ngrad, 1))
        mode = 1 if grads else 0
        wp = nat.dptr(w) if w is not None else None
        if timed:
            ms = ctypes.c_float()
            rc = self._lib.qfvm_batch_run_timed(self._h, mode, nat.dptr(vals), wp, nat.dptr(ev), nat.dptr(gr),
                                                ctypes.byref(ms))
        else:
            rc = self._lib.qfvm_batch_run(self._h, mode, nat.dptr(vals), wp, nat.dptr(ev), nat.dptr(gr))
        nat.check(rc, "batch run")
        exps, grs = [], []
        eo = go = 0
        for n, items, slots, nobs in self.groups:
            exps.append(ev[eo:eo + items * nobs].reshape(items, nobs))
            eo += items * nobs
            if grads:
                grs.append(gr[go:go + items * slots].reshape(items, slots))
            if self.grads:
                go += items * slots
        out = (exps, grs) if grads else (exps,)
        if timed:
            out = out + (float(ms.value),)
        return out if len(out) > 1 else out[0]

    def info(self) -> dict:
        ng, nv, ne, ngr = (ctypes.c_int64() for _ in range(4))
        kpr = (ctypes.c_int64 * 2)()
        gready = (ctypes.c_int32 * 2)()
        nat.check(self._lib.qfvm_batch_info(self._h, ctypes.byref(ng), ctypes.byref(nv), ctypes.byref(ne),
                                            ctypes.byref(ngr), kpr, gready), "batch info")
        return {"groups": ng.value, "values": nv.value, "expvals": ne.value, "grads": ngr.value,
                "kernels_per_run": [kpr[0], kpr[1]], "graph_ready": [bool(gready[0]), bool(gready[1])]}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.qfvm_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def group_passes(n: int, ops, precision="c64") -> tuple[int, int]:
    """(forward passes, reverse-sweep passes) of the plans a group runs
    (host planning only)."""
    lib = nat.load()
    gates = [o for o in ops if o.is_gate]
    arr, pool = ir.pack(gates)
    out = []
    for adjoint in (0, 1):
        h = ctypes.c_void_p()
        nat.check(lib.qfvm_plan_host_build_batched(int(n), _precision(precision), nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, adjoint,
                                                   ctypes.byref(h)), "host batched plan")
        counts = (ctypes.c_int64 * 4)()
        shape = (ctypes.c_int32 * 3)()
        nat.check(lib.qfvm_plan_host_counts(h, counts, shape))
        lib.qfvm_plan_destroy(h)
        out.append(int(counts[0]))
    return out[0], out[1]


def algorithmic_bytes(n: int, items: int, fwd_passes: int, rev_passes: int, amp_bytes: int = 8,
                      grads: bool = True) -> float:
    """HBM bytes a run of one group must move at least: zero-fill (write),
    forward passes (read + write), the expectation (read); with gradients
    lam = H psi (read + write) and reverse passes over psi and lam (2 x read +
    write)."""
    sn = float(amp_bytes) * items * (1 << n)
    b = sn + 2 * sn * fwd_passes + sn
    if grads:
        b += 2 * sn + 4 * sn * rev_passes
    return b
