"""Autotuner bookkeeping without a GPU: compiled shape lists, the process-wide
shape table the plans read, and the JSON cache round trip."""

import numpy as np
import pytest

import helpers
from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import autotune, workloads


def test_candidates_are_compiled_shapes():
    for prec in ("c128", "c64", "c128_ds"):
        for kind in autotune.KINDS:
            c = autotune.candidates(prec, kind)
            assert c, (prec, kind)
            assert autotune.current(prec, kind, 20) in c


def test_tuned_shape_reaches_the_planner():
    ops = workloads.random_layers(14, 4, seed=1)
    default = autotune.current("c64", 0, 14)
    other = next(s for s in autotune.candidates("c64", 0) if s != default and s[0] <= 14)
    try:
        autotune.set_shape("c64", 0, 14, other)
        assert autotune.current("c64", 0, 14) == other
        assert autotune.current("c64", 0, 15) == default  # per qubit count
        plan = helpers.host_plan(14, ops, precision=1)
        assert (plan["T"], plan["R"]) == other
    finally:
        autotune.set_shape("c64", 0, 14, None)
    assert autotune.current("c64", 0, 14) == default


def test_uncompiled_shape_is_refused():
    with pytest.raises(nat.QfvmError):
        autotune.set_shape("c128", 0, 20, (15, 2))
    with pytest.raises(nat.QfvmError):
        autotune.set_shape("c128", 1, 20, (13, 6))


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("QFVM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    shape = autotune.candidates("c64", 1)[-1]
    autotune._store("c64", 1, 17, shape, 1.5)
    try:
        assert autotune.apply_cached() == 1
        assert autotune.current("c64", 1, 17) == tuple(shape)
    finally:
        autotune.set_shape("c64", 1, 17, None)
