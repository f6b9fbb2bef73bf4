"""Device-resident statevector and compiled circuit plans (Python side).

``DeviceState`` owns one state in HBM (complex128 or complex64 storage);
``Plan`` is a circuit classified and fused once for a qubit count and
precision, runnable many times on device states.  Both are thin wrappers over
the C ABI in include/qfvm_gb300.h.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat
from . import ir


def _precision(p) -> int:
    if isinstance(p, str):
        if p not in nat.PRECISIONS:
            raise ValueError(f"unknown precision {p!r}")
        return nat.PRECISIONS[p]
    return int(p)


def pauli_masks(paulistr: str, pos) -> tuple[int, int, int]:
    """Flip mask (X and Y), Z mask (Z and Y) and Y count of a Pauli string
    (statevector.hpp:1252-1279)."""
    xm = zm = 0
    ny = 0
    for ch, q in zip(paulistr, pos):
        q = int(q)
        if ch == "X":
            xm |= 1 << q
        elif ch == "Y":
            xm |= 1 << q
            zm |= 1 << q
            ny += 1
        elif ch == "Z":
            zm |= 1 << q
        elif ch != "I":
            raise ValueError(f"unknown Pauli {ch!r}")
    return xm, zm, ny


def pack_terms(terms):
    """terms: iterable of (paulistr, pos) -> (x masks, z masks, y counts)."""
    xs, zs, ys = [], [], []
    for pstr, pos in terms:
        x, z, y = pauli_masks(pstr, pos)
        xs.append(x)
        zs.append(z)
        ys.append(y)
    return (np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64), np.array(ys, dtype=np.int32))


class DeviceState:
    """A statevector resident in GPU memory."""

    def __init__(self, num_qubits: int, precision="c128"):
        self._lib = nat.load()
        self.num_qubits = int(num_qubits)
        self.precision = _precision(precision)
        h = ctypes.c_void_p()
        nat.check(self._lib.qfvm_sv_create(self.num_qubits, self.precision, ctypes.byref(h)), "create state")
        self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def size(self) -> int:
        return 1 << self.num_qubits

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qfvm_sv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_zero(self):
        nat.check(self._lib.qfvm_sv_set_zero(self._h), "set_zero")
        return self

    def upload(self, psi: np.ndarray):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        nat.check(self._lib.qfvm_sv_upload(self._h, nat.dptr(psi.view(np.float64)), psi.size), "upload")
        return self

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.size, dtype=np.complex128)
        assert out.dtype == np.complex128 and out.flags.c_contiguous and out.size == self.size
        nat.check(self._lib.qfvm_sv_download(self._h, nat.dptr(out.view(np.float64)), out.size), "download")
        return out

    def apply(self, ops):
        arr, pool = ir.pack(ops)
        nat.check(self._lib.qfvm_sv_apply(self._h, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                                          pool.size), "apply")
        return self

    def expect(self, terms) -> np.ndarray:
        """Unweighted <P> for terms given as (paulistr, pos)."""
        x, z, y = pack_terms(terms)
        out = np.zeros(x.size, dtype=np.float64)
        if x.size:
            nat.check(self._lib.qfvm_sv_expect(self._h, nat.u64ptr(x), nat.u64ptr(z), nat.i32ptr(y), x.size,
                                               nat.dptr(out)), "expect")
        return out

    def sample(self, uniforms) -> np.ndarray:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        out = np.zeros(u.size, dtype=np.uint64)
        nat.check(self._lib.qfvm_sv_sample(self._h, nat.dptr(u), u.size, nat.u64ptr(out)), "sample")
        return out

    def sequential_blocks(self) -> int:
        """Blocks of 4096 amplitudes the last sample() summed element by
        element (the rest advanced the exact running sum by one integer
        addition each)."""
        v = ctypes.c_int64()
        nat.check(self._lib.qfvm_sv_sample_stats(self._h, ctypes.byref(v)), "sample stats")
        return v.value

    def norm2(self) -> float:
        v = ctypes.c_double()
        nat.check(self._lib.qfvm_sv_norm2(self._h, ctypes.byref(v)), "norm2")
        return v.value

    def device_ptr(self) -> tuple[int, int]:
        p = ctypes.c_void_p()
        nb = ctypes.c_uint64()
        nat.check(self._lib.qfvm_sv_device_ptr(self._h, ctypes.byref(p), ctypes.byref(nb)), "device_ptr")
        return int(p.value or 0), int(nb.value)

    def stream(self) -> int:
        s = ctypes.c_void_p()
        nat.check(self._lib.qfvm_sv_stream(self._h, ctypes.byref(s)), "stream")
        return int(s.value or 0)


class Plan:
    """A circuit classified and fused for (num_qubits, precision)."""

    def __init__(self, num_qubits: int, ops, precision="c128", tile_qubits: int = 0, reg_qubits: int = 0):
        self._lib = nat.load()
        self.num_qubits = int(num_qubits)
        self.precision = _precision(precision)
        arr, pool = ir.pack(ops)
        self._keep = (arr, pool)
        h = ctypes.c_void_p()
        nat.check(self._lib.qfvm_plan_create(self.num_qubits, self.precision, nat.vptr(arr), arr.size,
                                             nat.dptr(pool.view(np.float64)), pool.size, int(tile_qubits),
                                             int(reg_qubits), ctypes.byref(h)), "plan")
        self._h = h

    def stats(self) -> dict:
        p, r, g = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        pb, gb = ctypes.c_double(), ctypes.c_double()
        nat.check(self._lib.qfvm_plan_stats(self._h, ctypes.byref(p), ctypes.byref(r), ctypes.byref(g),
                                            ctypes.byref(pb), ctypes.byref(gb)), "plan stats")
        return {"passes": p.value, "rounds": r.value, "gates": g.value, "pass_bytes": pb.value,
                "gate_bytes": gb.value}

    def run(self, state: DeviceState):
        """Enqueue the plan on the state's stream (asynchronous)."""
        nat.check(self._lib.qfvm_plan_run(self._h, state.handle), "plan run")

    def run_timed(self, state: DeviceState) -> tuple[np.ndarray, np.ndarray]:
        """Run with CUDA events around every pass; returns (ms per pass, pass type)."""
        npass = self.stats()["passes"]
        ms = np.zeros(npass, dtype=np.float32)
        ty = np.zeros(npass, dtype=np.int32)
        nat.check(self._lib.qfvm_plan_run_timed(self._h, state.handle, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                nat.i32ptr(ty)), "plan run (timed)")
        return ms, ty

    def jit_passes(self, nstates: int = 1) -> int:
        """Passes of this plan that run as circuit-specialised kernels (known
        after the first run)."""
        c = ctypes.c_int64()
        nat.check(self._lib.qfvm_jit_plan_passes(self._h, int(nstates), ctypes.byref(c)), "plan jit passes")
        return c.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qfvm_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def jit_configure(enabled: bool = True, nb_one: int = 2, minb_one: int = 0, nb_two: int = 1, minb_two: int = 0):
    """Circuit-specialised tile passes: on/off, and the tile buffers / minimum
    resident CTAs per SM of one-state and two-state passes (0 = automatic).
    Applies to plans prepared afterwards."""
    nat.check(nat.load().qfvm_jit_configure(int(bool(enabled)), int(nb_one), int(minb_one), int(nb_two),
                                            int(minb_two)), "jit configure")


def jit_config() -> dict:
    c = (ctypes.c_int32 * 5)()
    nat.check(nat.load().qfvm_jit_get_config(c), "jit config")
    return {"enabled": bool(c[0]), "nb_one": c[1], "minb_one": c[2], "nb_two": c[3], "minb_two": c[4]}
