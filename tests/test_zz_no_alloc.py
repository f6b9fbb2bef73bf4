"""The allocation-free expectation entry point (qfvm_expect_device_noalloc).

It serves callers that cannot allocate GPU memory while running (a process
whose HBM is reserved up front by its own pool, or a hot loop where
cudaMalloc/cudaFree would synchronise the device): the caller passes a state
already in its own device memory, and the library uses a fixed 64 KiB scratch
array instead of allocating.  This file is collected last on purpose.

The checks: through the C ABI, the allocation-free call gives the same values
as the existing qfvm_sv_expect entry point and as the oracle's expect_pauli
on the same state, within the tests' tolerances, on two calls in a row (the
second with a different, smaller term set, so stale scratch contents would
show); the device's free memory does not move across repeated calls; and it
rejects a request above its stated limit and a state pointer that is not
device memory, before launching anything.
"""

import ctypes

import numpy as np
import pytest

import helpers
import oracle
from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import engine

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 1e-6


def _terms(n, seed, count):
    rng = np.random.default_rng(seed)
    terms = []
    for _ in range(count):
        k = int(rng.integers(1, 4))
        qs = [int(q) for q in rng.choice(n, k, replace=False)]
        terms.append(("".join(rng.choice(list("XYZ"), k)), qs))
    terms.append(("Z", [0]))
    return terms


def _noalloc(lib, st, terms, precision):
    ptr, _ = st.device_ptr()
    x, z, y = engine.pack_terms(terms)
    out = np.full(len(terms), np.nan)
    rc = lib.qfvm_expect_device_noalloc(ctypes.c_void_p(ptr), st.size, precision, nat.u64ptr(x), nat.u64ptr(z),
                                        nat.i32ptr(y), len(terms), nat.dptr(out), ctypes.c_void_p(st.stream()))
    assert rc == 0, lib.qfvm_noalloc_last_error()
    return out


@pytest.mark.parametrize("precision,tol", [(nat.QFVM_C128, TOL128), (nat.QFVM_C64, TOL64)])
def test_noalloc_matches_existing_entry_point(precision, tol):
    from pyquafu_gb300.builder import build

    build()
    lib = nat.load()
    n = 16
    psi = helpers.random_state(n, 42)
    st = engine.DeviceState(n, "c64" if precision == nat.QFVM_C64 else "c128")
    st.upload(psi)
    if precision == nat.QFVM_C64:
        psi = psi.astype(np.complex64).astype(np.complex128)  # what the complex64 state holds
    first = _terms(n, 1, 30)
    second = _terms(n, 2, 7)
    for terms in (first, second):  # two calls in a row
        got = _noalloc(lib, st, terms, precision)
        ref = st.expect(terms)
        np.testing.assert_allclose(got, ref, atol=tol, rtol=0)
        exact = [oracle.expect_pauli(psi, p, pos) for p, pos in terms]
        np.testing.assert_allclose(got, exact, atol=tol, rtol=0)
    st.close()


def test_noalloc_leaves_device_memory_untouched():
    import torch

    lib = nat.load()
    n = 18
    st = engine.DeviceState(n, "c128")
    st.upload(helpers.random_state(n, 7))
    terms = _terms(n, 3, 40)
    _noalloc(lib, st, terms, nat.QFVM_C128)  # first call: module and scratch address set up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        _noalloc(lib, st, terms, nat.QFVM_C128)
    free1 = torch.cuda.mem_get_info()[0]
    st.close()
    assert free1 == free0


def test_noalloc_rejects_host_pointer():
    lib = nat.load()
    host = np.zeros(2 * 16, dtype=np.float64)  # 16 complex128 amplitudes in host memory
    x = np.zeros(1, dtype=np.uint64)
    z = np.ones(1, dtype=np.uint64)
    y = np.zeros(1, dtype=np.int32)
    out = np.zeros(1)
    rc = lib.qfvm_expect_device_noalloc(ctypes.c_void_p(host.ctypes.data), 16, nat.QFVM_C128, nat.u64ptr(x),
                                        nat.u64ptr(z), nat.i32ptr(y), 1, nat.dptr(out), None)
    assert rc == 1
    assert b"device memory" in lib.qfvm_noalloc_last_error()


def test_noalloc_rejects_oversize_request():
    lib = nat.load()
    st = engine.DeviceState(4, "c128").set_zero()
    ptr, _ = st.device_ptr()
    count = 1025
    x = np.zeros(count, dtype=np.uint64)
    z = np.ones(count, dtype=np.uint64)
    y = np.zeros(count, dtype=np.int32)
    out = np.zeros(count)
    rc = lib.qfvm_expect_device_noalloc(ctypes.c_void_p(ptr), st.size, nat.QFVM_C128, nat.u64ptr(x), nat.u64ptr(z),
                                        nat.i32ptr(y), count, nat.dptr(out), None)
    assert rc == 1
    assert b"1024" in lib.qfvm_noalloc_last_error()
    st.close()
