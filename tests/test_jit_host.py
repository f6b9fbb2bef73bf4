"""The PTX generator of circuit-specialised tile passes, on the CPU: every
tile pass of representative plans (complex128 and complex64 one-state
passes, double-single passes, reverse sweeps with probes, batched plans)
is emitted, and where the
toolkit's ptxas is on the PATH it must assemble for sm_103a (and compile
through the library's own PTX compiler path); passes the
generator does not handle are reported as unsupported, not emitted."""

import ctypes
import shutil
import subprocess

import numpy as np
import pytest

import helpers
from pyquafu_gb300 import _native as nat
from pyquafu_gb300 import ir, workloads


def plan_handle(n, ops, precision, T=0, R=0, batched=False, adjoint=False):
    lib = nat.load()
    arr, pool = ir.pack(ops)
    h = ctypes.c_void_p()
    if batched:
        nat.check(lib.qfvm_plan_host_build_batched(n, precision, nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, int(adjoint),
                                                   ctypes.byref(h)))
    else:
        nat.check(lib.qfvm_plan_host_build(n, precision, nat.vptr(arr), arr.size, nat.dptr(pool.view(np.float64)),
                                           pool.size, T, R, ctypes.byref(h)))
    return h


def pass_ptx(h, i, nstates):
    lib = nat.load()
    ln = ctypes.c_int64()
    rc = lib.qfvm_jit_pass_ptx(h, i, nstates, None, 0, ctypes.byref(ln))
    if rc != 0:
        return None
    buf = ctypes.create_string_buffer(ln.value + 1)
    nat.check(lib.qfvm_jit_pass_ptx(h, i, nstates, buf, ln.value + 1, ctypes.byref(ln)))
    return buf.value.decode()


def assemble(tmp_path, src, tag):
    exe = shutil.which("ptxas")
    if exe is None:
        return
    f = tmp_path / f"{tag}.ptx"
    f.write_text(src)
    r = subprocess.run([exe, "-arch=sm_103a", "-O1", "-o", str(tmp_path / f"{tag}.cubin"), str(f)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]


CASES = [
    ("c128_11_3", 16, 0, 11, 3, False, False, 1),
    ("c128_12_5", 16, 0, 12, 5, False, False, 1),
    ("c64_13_4", 16, 1, 13, 4, False, False, 1),
    ("ds_12_3", 16, 2, 12, 3, False, False, 1),
    ("c64_rev_batched", 16, 1, 0, 0, True, True, 2),
    ("c128_rev_batched", 15, 0, 0, 0, True, True, 2),
    ("c64_fwd_batched", 16, 1, 0, 0, True, False, 1),
]


@pytest.mark.parametrize("tag,n,precision,T,R,batched,adjoint,nstates", CASES)
def test_passes_assemble(tmp_path, tag, n, precision, T, R, batched, adjoint, nstates):
    if batched:
        ops, _, _, _ = workloads.qnn_batch(batch=2, n=n, layers=2, seed=1)
    else:
        ops = workloads.random_layers(n, 4, seed=n + T, extras=True)
    h = plan_handle(n, ops, precision, T, R, batched, adjoint)
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(nat.load().qfvm_plan_host_counts(h, counts, shape))
    passes = np.zeros(counts[0], helpers.PASS_DT)
    nat.check(nat.load().qfvm_plan_host_copy(h, nat.vptr(passes), None, None, None))
    emitted = 0
    for i in range(counts[0]):
        src = pass_ptx(h, i, nstates)
        if int(passes[i]["type"]) != helpers.PASS_TILE:
            assert src is None
            continue
        assert src is not None and ".target sm_103a" in src
        emitted += 1
        if i == counts[0] - 1:
            assemble(tmp_path, src, f"{tag}_{i}")
        if i == 0:
            info = ctypes.create_string_buffer(4096)
            rc = nat.load().qfvm_jit_pass_compile(h, i, nstates, info, 4096)
            assert rc == 0, info.value.decode()
    nat.load().qfvm_plan_destroy(h)
    assert emitted > 0


def dense2_circuit(n, seed):
    """Random two-qubit unitaries (shared-memory steps of tile passes) between
    layers of one-qubit gates and cx."""
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(4):
        ops += workloads.random_layers(n, 1, seed=seed * 10 + layer)
        for _ in range(3):
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
            u, _ = np.linalg.qr(z)
            ops.append(workloads.matrix_gate("u2", (a, b), u))
    return ops


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_shared_memory_steps_assemble(tmp_path, precision):
    n = 16
    T, R = (12, 4) if precision == 1 else (11, 4)
    h = plan_handle(n, dense2_circuit(n, 3), precision, T, R)
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(nat.load().qfvm_plan_host_counts(h, counts, shape))
    steps = np.zeros(counts[1], helpers.STEP_DT)
    nat.check(nat.load().qfvm_plan_host_copy(h, None, nat.vptr(steps), None, None))
    assert (steps["type"] == helpers.STEP_SMEM).any()
    for i in range(counts[0]):
        src = pass_ptx(h, i, 1)
        assert src is not None
        if i == 0:
            assemble(tmp_path, src, f"smem_{precision}")
    nat.load().qfvm_plan_destroy(h)


def test_probe_pass_needs_two_states():
    ops, _, _, _ = workloads.qnn_batch(batch=2, n=16, layers=2, seed=1)
    h = plan_handle(16, ops, 1, batched=True, adjoint=True)
    assert pass_ptx(h, 0, 1) is None  # probes read lam
    assert pass_ptx(h, 0, 2) is not None
    nat.load().qfvm_plan_destroy(h)


def test_jit_config_roundtrip():
    from pyquafu_gb300 import engine

    engine.jit_configure(True, 2, 1, 1, 2)
    assert engine.jit_config() == {"enabled": True, "nb_one": 2, "minb_one": 1, "nb_two": 1, "minb_two": 2}
    with pytest.raises(nat.QfvmError):
        engine.jit_configure(True, 3, 0, 1, 0)
    engine.jit_configure(True)


def test_pass_text_depends_on_structure_only():
    """The module cache keys passes by structure: the same circuit with other
    rotation angles emits identical PTX (coefficients are loaded, not baked
    in); moving a gate to another qubit changes it."""
    n = 16
    a = workloads.hea(n, 2, seed=1)[0]
    b = workloads.hea(n, 2, seed=2)[0]  # same structure, other angles
    c = list(a)
    c[0] = workloads.named("ry", ((c[0].qubits[0] + 1) % n,), c[0].params)
    texts = []
    for ops in (a, b, c):
        h = plan_handle(n, ops, 1, 12, 4)
        texts.append(pass_ptx(h, 0, 1))
        nat.load().qfvm_plan_destroy(h)
    assert texts[0] == texts[1]
    assert texts[0] != texts[2]


@pytest.mark.parametrize("precision,T,R,nstates,adjoint", [(1, 12, 4, 1, False), (2, 12, 3, 1, False),
                                                           (0, 11, 4, 1, False), (0, 11, 4, 2, True)])
def test_bounds_checked_passes(tmp_path, monkeypatch, precision, T, R, nstates, adjoint):
    """QFVM_BOUNDS_CHECK=1: every shared-memory access, global store and bulk
    copy of a specialised pass is predicated on a range check whose failure
    writes QFVM_ERR_BOUNDS (7) to the status word; the passes assemble."""
    monkeypatch.setenv("QFVM_BOUNDS_CHECK", "1")
    n = 16
    ops = workloads.random_layers(n, 4, seed=9, extras=True)
    ops.append(workloads.matrix_gate("u2", (3, 9), np.eye(4)))  # a shared-memory step
    if adjoint:
        ops, _ = workloads.hea(n, 2, seed=1)
        h = plan_handle(n, ops, precision, adjoint=True, batched=True)
    else:
        h = plan_handle(n, ops, precision, T, R)
    checked = 0
    for i in range(16):
        src = pass_ptx(h, i, nstates)
        if src is None:
            continue
        for line in src.splitlines():
            ins = line.strip()
            body = ins.split(" ", 1)[1] if ins.startswith("@") else ins
            if body.startswith(("ld.shared", "st.shared", "st.global.cs", "cp.async.bulk.shared::cluster.global",
                                "cp.async.bulk.global.shared::cta")):
                assert ins.startswith("@"), ins
                checked += 1
        assert "atom.global.cas.b32" in src and ", 0, 7;" in src
        assemble(tmp_path, src, f"bc{precision}_{i}")
    assert checked > 0


def test_double_single_chain_pattern(tmp_path):
    """A double-single plan of several specialised passes hands the state on
    as float pairs: the first pass converts FP64 at staging and writes pairs
    with bulk stores, the middle passes neither convert nor store per thread,
    the last converts back and stores FP64 per thread.  Every pass assembles."""
    n = 18
    ops = workloads.random_layers(n, 6, seed=3, extras=True)
    h = plan_handle(n, ops, 2, 12, 3)
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(nat.load().qfvm_plan_host_counts(h, counts, shape))
    npass = int(counts[0])
    assert npass >= 3
    srcs = [pass_ptx(h, i, 1) for i in range(npass)]
    assert all(s is not None for s in srcs)
    for i, src in enumerate(srcs):
        converts_in = "ld.shared.v2.f64" in src
        stores_fp64 = "st.global.cs.v2.f64" in src
        bulk_out = "cp.async.bulk.global.shared" in src
        assert converts_in == (i == 0), i
        assert stores_fp64 == (i == npass - 1), i
        assert bulk_out == (i < npass - 1), i
        assemble(tmp_path, src, f"chain{i}")


def test_no_chain_across_a_global_pass():
    """A double-single plan with a pass that is not a tile pass (a dense gate
    on eight targets runs as its own global pass, which reads FP64) keeps
    FP64 between all passes: every tile pass converts at staging and stores
    FP64, none writes float pairs."""
    n = 18
    rng = np.random.default_rng(2)
    u, _ = np.linalg.qr(rng.normal(size=(256, 256)) + 1j * rng.normal(size=(256, 256)))
    ops = workloads.random_layers(n, 3, seed=4) + [workloads.matrix_gate("u8", tuple(range(2, 10)), u)]
    ops += workloads.random_layers(n, 3, seed=5)
    h = plan_handle(n, ops, 2, 12, 3)
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(nat.load().qfvm_plan_host_counts(h, counts, shape))
    passes = np.zeros(counts[0], helpers.PASS_DT)
    nat.check(nat.load().qfvm_plan_host_copy(h, nat.vptr(passes), None, None, None))
    assert any(int(p["type"]) != 0 for p in passes)
    tiles = 0
    for i, p in enumerate(passes):
        if int(p["type"]) != 0:
            continue
        src = pass_ptx(h, i, 1)
        assert "ld.shared.v2.f64" in src and "st.global.cs.v2.f64" in src
        assert "cp.async.bulk.global.shared" not in src
        tiles += 1
    assert tiles >= 2


def ptx_instructions(src):
    """Instruction statements of a PTX text (no directives, labels or comments)."""
    k = 0
    for ln in src.split("\n"):
        t = ln.strip()
        if t and not t.startswith(("//", ".")) and not t.endswith(":") and t not in ("{", "}") and t.endswith(";"):
            k += 1
    return k


@pytest.mark.parametrize("precision,adjoint,median_max,max_max", [
    (2, True, 18000, 60000),   # float-pair reverse sweep at (11, 3): 14.3 K / 50.2 K
    (0, True, 8000, 24000),    # FP64 reverse sweep at (11, 4): 4.7 K / 15.2 K
    (1, True, 8000, 24000),    # complex64 reverse sweep at (12, 4): 4.5 K / 16.3 K
    (2, False, 6000, 9000),    # float-pair pass at (12, 3): 3.8 K / 6.0 K
    (1, False, 5000, 7000),    # complex64 pass at (13, 5): 3.0 K / 4.5 K
])
def test_specialised_pass_code_size(precision, adjoint, median_max, max_max):
    """Code size of the default specialised passes on the benchmark circuits
    (24-qubit HEA gradient, 30-qubit random layers): the float-pair reverse
    sweep at four register qubits emitted a median of 27 K instructions per
    pass and stalled on instruction fetch on the GPU; the bounds keep the
    defaults well below that."""
    lib = nat.load()
    if adjoint:
        n = 24
        ops, _ = workloads.hea(n, 20, seed=0)
        arr, pool = ir.pack(ops)
        h = ctypes.c_void_p()
        nat.check(lib.qfvm_plan_host_build_adjoint(n, precision, nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, ctypes.byref(h)))
    else:
        n = 30
        h = plan_handle(n, workloads.random_layers(n, 40, seed=0, extras=True), precision)
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(lib.qfvm_plan_host_counts(h, counts, shape))
    nstates = 2 if adjoint else 1
    sizes = [ptx_instructions(s) for s in (pass_ptx(h, i, nstates) for i in range(counts[0])) if s]
    lib.qfvm_plan_destroy(h)
    assert len(sizes) >= 40
    assert np.median(sizes) <= median_max and max(sizes) <= max_max, (tuple(shape), np.median(sizes), max(sizes))


def default_plan(precision, adjoint):
    """Host plan of a benchmark circuit at the default shape: the 24-qubit
    HEA gradient's reverse sweep, or the 30-qubit random-layer circuit."""
    lib = nat.load()
    if adjoint:
        ops, _ = workloads.hea(24, 20, seed=0)
        arr, pool = ir.pack(ops)
        h = ctypes.c_void_p()
        nat.check(lib.qfvm_plan_host_build_adjoint(24, precision, nat.vptr(arr), arr.size,
                                                   nat.dptr(pool.view(np.float64)), pool.size, ctypes.byref(h)))
        return h
    return plan_handle(30, workloads.random_layers(30, 40, seed=0, extras=True), precision)


# (arithmetic, reverse sweep): threads per CTA and resident CTAs per SM of the
# automatic register budget (128 registers; 80 for complex64 one-state passes;
# 255 when a round's amplitudes alone need more than 64)
RESIDENCY = {(0, False): (128, 4), (1, False): (256, 3), (2, False): (512, 1),
             (0, True): (128, 2), (1, True): (256, 2), (2, True): (256, 2)}


@pytest.mark.parametrize("precision,adjoint", sorted(RESIDENCY))
def test_host_ptx_carries_device_residency(precision, adjoint):
    """The host-side PTX query reports the pass the device path compiles:
    its launch bounds are the automatic register budget's."""
    h = default_plan(precision, adjoint)
    src = pass_ptx(h, 0, 2 if adjoint else 1)
    nat.load().qfvm_plan_destroy(h)
    nt, minb = RESIDENCY[(precision, adjoint)]
    assert f".maxntid {nt}, 1, 1" in src and f".minnctapersm {minb}\n" in src


@pytest.mark.parametrize("precision,adjoint,spill_max", [
    (2, False, 0),     # the float-pair pass of the headline: no local memory
    (0, False, 64), (1, False, 64),
    (0, True, 128), (1, True, 192), (2, True, 384),
])
def test_largest_passes_fit_their_register_budget(precision, adjoint, spill_max):
    """The two largest default passes of each benchmark circuit compiled for
    sm_103a on the host: registers within the launch bounds' budget and
    spill traffic bounded (bytes of spill loads per thread)."""
    import re

    lib = nat.load()
    h = default_plan(precision, adjoint)
    nstates = 2 if adjoint else 1
    counts = (ctypes.c_int64 * 4)()
    shape = (ctypes.c_int32 * 3)()
    nat.check(lib.qfvm_plan_host_counts(h, counts, shape))
    sizes = sorted(((ptx_instructions(pass_ptx(h, i, nstates) or ""), i) for i in range(counts[0])), reverse=True)
    nt, minb = RESIDENCY[(precision, adjoint)]
    budget = min(255, 65536 // (nt * minb))
    try:
        for _, i in sizes[:2]:
            info = ctypes.create_string_buffer(8192)
            nat.check(lib.qfvm_jit_pass_compile(h, i, nstates, info, 8192))
            log = info.value.decode()
            regs = re.findall(r"Used (\d+) registers", log)
            if not regs:
                pytest.skip("the PTX compiler library is not linked in: no compile log on the host")
            assert int(regs[0]) <= budget, (i, log)
            spill = re.findall(r"(\d+) bytes spill loads", log)
            assert spill and int(spill[0]) <= spill_max, (i, log)
    finally:
        lib.qfvm_plan_destroy(h)
