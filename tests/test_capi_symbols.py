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
