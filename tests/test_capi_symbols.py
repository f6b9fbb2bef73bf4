"""The C-ABI library loads and exports every symbol include/*.h declares
(no compute calls)."""

import ctypes
import glob
import os
import re

import pytest

from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import builder as bld

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*\*?\s+\**(qfvm_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    bld.build()
    return nat.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(nat.PROTOTYPES) <= set(names)


def test_abi_version(lib):
    assert lib.qfvm_abi_version() == 1


def test_launch_counter_readable(lib):
    assert lib.qfvm_launch_count() >= 0


def test_no_device_is_an_error_not_a_crash(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.qfvm_sv_create(4, 0, ctypes.byref(h))
    assert rc == 6
    assert b"CUDA" in lib.qfvm_last_error()


COMPILED_SHAPES = {  # (arithmetic, pass kind): the (tile qubits, register qubits) the library instantiates
    (nat.QFVM_C128, 0): {(11, 4), (12, 4), (12, 5), (12, 3), (11, 3)},
    (nat.QFVM_C64, 0): {(12, 5), (13, 5), (12, 4), (13, 4)},
    (nat.QFVM_C128_DS, 0): {(11, 4), (12, 4), (12, 5), (12, 3)},
    (nat.QFVM_C128, 1): {(11, 4), (11, 3)},
    (nat.QFVM_C64, 1): {(12, 4), (11, 4), (13, 4)},
    (nat.QFVM_C128_DS, 1): {(11, 4), (12, 3), (11, 3)},
}
DEFAULT_SHAPES = {  # one-state passes, then the adjoint's two-state reverse sweep
    (nat.QFVM_C128, 0): (11, 4), (nat.QFVM_C64, 0): (13, 5), (nat.QFVM_C128_DS, 0): (12, 3),
    (nat.QFVM_C128, 1): (11, 4), (nat.QFVM_C64, 1): (12, 4), (nat.QFVM_C128_DS, 1): (11, 3),
}


def test_compiled_shape_table(lib):
    """The shapes each arithmetic's translation units instantiate (host
    queries only), and the built-in defaults are among them."""
    for (prec, kind), want in COMPILED_SHAPES.items():
        got = {(t, r) for t in range(6, 16) for r in range(1, 8) if lib.qfvm_shape_supported(prec, kind, t, r)}
        assert got == want, (prec, kind)
    assert lib.qfvm_shape_supported(7, 0, 11, 4) == 0 and lib.qfvm_shape_supported(nat.QFVM_C128, 2, 11, 4) == 0
    t, r = ctypes.c_int32(), ctypes.c_int32()
    for (prec, kind), want in DEFAULT_SHAPES.items():
        for n in (20, 24, 30):
            assert lib.qfvm_set_tuned_shape(prec, kind, n, 0, 0) == 0  # the built-in default, not a tuned one
            assert lib.qfvm_get_shape(prec, kind, n, ctypes.byref(t), ctypes.byref(r)) == 0
            assert (t.value, r.value) == want, (prec, kind, n)


def test_python_constants_match_header():
    """The ctypes layer's status codes, arithmetic kinds and limits are the
    header's, and every status code the header declares has a name."""
    text = open(os.path.join(ROOT, "include", "qfvm_gb300.h")).read()
    defined = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(QFVM_[A-Z0-9_]+)\s+(\d+)", text)}
    enums = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(QFVM_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    header = {**defined, **enums}
    names = [n for n in dir(nat) if n.startswith("QFVM_") and isinstance(getattr(nat, n), int)]
    assert len(names) >= 12
    for n in names:
        assert n in header, n
        assert getattr(nat, n) == header[n], n
    for n, v in header.items():
        if n.startswith("QFVM_ERR_"):
            assert v in nat.STATUS, n
