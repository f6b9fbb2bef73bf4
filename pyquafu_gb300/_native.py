"""ctypes binding of the engine's C ABI (include/qfvm_gb300.h).

The shared library is built in-tree by ``pyquafu_gb300.build``.  There is no
CPU fallback: if the library is missing or cannot be loaded, every entry point
raises ``QfvmError``.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .builder import LIB

QFVM_C128, QFVM_C64, QFVM_C128_DS = 0, 1, 2
PRECISIONS = {"c128": QFVM_C128, "complex128": QFVM_C128, "c64": QFVM_C64, "complex64": QFVM_C64,
              "c128_ds": QFVM_C128_DS}

QFVM_ERR_INVALID, QFVM_ERR_CUDA, QFVM_ERR_NOMEM, QFVM_ERR_UNSUPPORTED, QFVM_ERR_TIMEOUT, QFVM_ERR_NODEVICE, \
    QFVM_ERR_BOUNDS = range(1, 8)

QFVM_MAX_QUBITS = 34     # largest state the engine plans (2^34 amplitudes)
QFVM_MAX_OP_QUBITS = 16  # most qubits (targets and controls) of one operation

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
    4: "unsupported", 5: "device wait timed out", 6: "no CUDA device", 7: "index out of bounds",
}


class QfvmError(RuntimeError):
    """Error raised by the GB300 engine (carries the C status code)."""

    def __init__(self, msg: str, status: int = 1):
        super().__init__(msg)
        self.status = status


_lib = None
_lock = threading.Lock()

c_dp = ctypes.POINTER(ctypes.c_double)
c_u64p = ctypes.POINTER(ctypes.c_uint64)
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_vp = ctypes.c_void_p

# name -> (restype, argtypes)
PROTOTYPES = {
    "qfvm_last_error": (ctypes.c_char_p, []),
    "qfvm_abi_version": (ctypes.c_int32, []),
    "qfvm_launch_count": (ctypes.c_uint64, []),
    "qfvm_simulate_circuit": (ctypes.c_int, [ctypes.c_int32, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64, c_dp,
                                             ctypes.c_int32, c_dp, ctypes.c_int64, c_u64p]),
    "qfvm_applyop_statevec": (ctypes.c_int, [c_vp, c_dp, ctypes.c_int64, c_dp, ctypes.c_uint64]),
    "qfvm_sampling_statevec": (ctypes.c_int, [c_dp, ctypes.c_uint64, c_dp, ctypes.c_int64, c_u64p]),
    "qfvm_expect_statevec": (ctypes.c_int, [c_dp, ctypes.c_uint64, c_u64p, c_u64p, c_i32p, ctypes.c_int64, c_dp]),
    "qfvm_expect_device_noalloc": (ctypes.c_int, [c_vp, ctypes.c_uint64, ctypes.c_int32, c_u64p, c_u64p, c_i32p,
                                                  ctypes.c_int64, c_dp, c_vp]),
    "qfvm_noalloc_last_error": (ctypes.c_char_p, []),
    "qfvm_test_fault": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64]),
    "qfvm_set_c128_arithmetic": (ctypes.c_int, [ctypes.c_int32]),
    "qfvm_get_c128_arithmetic": (ctypes.c_int32, []),
    "qfvm_simulate_shots": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp,
                                           ctypes.c_int64, c_dp, ctypes.c_int64, c_dp, ctypes.c_int64, c_u64p, c_dp]),
    "qfvm_simulate_noise": (ctypes.c_int, [ctypes.c_int32, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64, c_dp,
                                           ctypes.c_int64, c_dp, ctypes.c_int64, c_u64p, c_u64p, c_u64p, c_i32p,
                                           c_dp, ctypes.c_int64, c_dp]),
    "qfvm_adjoint": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64,
                                    c_u64p, c_u64p, c_i32p, c_dp, ctypes.c_int64, c_dp, c_dp, c_dp, ctypes.c_int64]),
    "qfvm_sv_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    "qfvm_sv_destroy": (ctypes.c_int, [c_vp]),
    "qfvm_sv_set_zero": (ctypes.c_int, [c_vp]),
    "qfvm_sv_upload": (ctypes.c_int, [c_vp, c_dp, ctypes.c_uint64]),
    "qfvm_sv_download": (ctypes.c_int, [c_vp, c_dp, ctypes.c_uint64]),
    "qfvm_sv_apply": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64]),
    "qfvm_sv_expect": (ctypes.c_int, [c_vp, c_u64p, c_u64p, c_i32p, ctypes.c_int64, c_dp]),
    "qfvm_sv_sample": (ctypes.c_int, [c_vp, c_dp, ctypes.c_int64, c_u64p]),
    "qfvm_sv_norm2": (ctypes.c_int, [c_vp, c_dp]),
    "qfvm_sv_sample_stats": (ctypes.c_int, [c_vp, ctypes.POINTER(ctypes.c_int64)]),
    "qfvm_sv_device_ptr": (ctypes.c_int, [c_vp, ctypes.POINTER(c_vp), c_u64p]),
    "qfvm_sv_stream": (ctypes.c_int, [c_vp, ctypes.POINTER(c_vp)]),
    "qfvm_plan_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    "qfvm_plan_destroy": (ctypes.c_int, [c_vp]),
    "qfvm_plan_stats": (ctypes.c_int, [c_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), c_dp, c_dp]),
    "qfvm_plan_run": (ctypes.c_int, [c_vp, c_vp]),
    "qfvm_plan_run_timed": (ctypes.c_int, [c_vp, c_vp, ctypes.POINTER(ctypes.c_float), c_i32p]),
    "qfvm_batch_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_i32p, ctypes.POINTER(c_vp)]),
    "qfvm_shape_supported": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "qfvm_set_tuned_shape": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_int32]),
    "qfvm_get_shape": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, c_i32p, c_i32p]),
    "qfvm_batch_add_group": (ctypes.c_int, [c_vp, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp, ctypes.c_int64,
                                            c_u64p, c_u64p, c_i32p, c_dp, c_i32p, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_int64]),
    "qfvm_batch_run": (ctypes.c_int, [c_vp, ctypes.c_int32, c_dp, c_dp, c_dp, c_dp]),
    "qfvm_batch_run_timed": (ctypes.c_int, [c_vp, ctypes.c_int32, c_dp, c_dp, c_dp, c_dp,
                                            ctypes.POINTER(ctypes.c_float)]),
    "qfvm_batch_info": (ctypes.c_int, [c_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), c_i32p]),
    "qfvm_batch_destroy": (ctypes.c_int, [c_vp]),
    "qfvm_plan_host_build": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp,
                                            ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    "qfvm_plan_host_counts": (ctypes.c_int, [c_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]),
    "qfvm_plan_host_build_adjoint": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp,
                                                    ctypes.c_int64, ctypes.POINTER(c_vp)]),
    "qfvm_plan_host_build_batched": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, c_vp, ctypes.c_int64, c_dp,
                                                    ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    "qfvm_plan_host_binds": (ctypes.c_int, [c_vp, ctypes.POINTER(ctypes.c_int64), c_i32p]),
    "qfvm_plan_host_probe_slots": (ctypes.c_int, [c_vp, c_i32p]),
    "qfvm_plan_host_copy": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_dp]),
    "qfvm_jit_configure": (ctypes.c_int, [ctypes.c_int32] * 5),
    "qfvm_jit_get_config": (ctypes.c_int, [c_i32p]),
    "qfvm_jit_pass_ptx": (ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int64,
                                         ctypes.POINTER(ctypes.c_int64)]),
    "qfvm_jit_plan_passes": (ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]),
    "qfvm_jit_pass_compile": (ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int64]),
}


def load(path: str | None = None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB
        if not os.path.exists(path):
            raise QfvmError(f"GB300 engine library not built: {path} (run pyquafu_gb300.builder.build())", 6)
        try:
            lib = ctypes.CDLL(path)
        except OSError as exc:
            raise QfvmError(f"cannot load the GB300 engine library {path}: {exc}", 6) from exc
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().qfvm_last_error().decode("utf-8", "replace")
        raise QfvmError(f"{what}: {STATUS.get(rc, rc)}: {msg}" if what else f"{STATUS.get(rc, rc)}: {msg}", rc)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(c_dp)


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(c_u64p)


def i32ptr(a: np.ndarray):
    return a.ctypes.data_as(c_i32p)


def vptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def launch_count() -> int:
    return int(load().qfvm_launch_count())
