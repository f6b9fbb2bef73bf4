"""Build the engine's shared library in-tree (nvcc, sm_103a only).

Produces ``pyquafu_gb300/_lib/libqfvm_gb300.so`` from ``csrc/``: each
translation unit is compiled in parallel, then linked with the host planner.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libqfvm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# CUDA and host translation units, longest compiles first (the float-pair and
# two-state instantiations, then the PTX generator), so that the parallel
# build is not left waiting on one of them at the end
SOURCES = ["adjoint_ds_r4.cu", "pass_ds_r5.cu", "adjoint_ds.cu", "pass_ds.cu", "adjoint_c64.cu", "pass_c128.cu",
           "pass_c64.cu", "adjoint_c128.cu", "jit_ptx.cpp", "kernels.cu", "plan.cpp", "adjoint.cu", "batch.cu",
           "shots.cu", "noise.cu", "sample.cu", "capi.cu", "batch_capi.cu", "shots_capi.cu", "noise_capi.cu",
           "noalloc.cu", "jit.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def ptx_compiler_lib():
    """The toolkit's static PTX compiler library (parallel compilation of
    circuit-specialised passes), or None: the driver then compiles them."""
    home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        f = os.path.join(home, sub, "libnvptxcompiler_static.a")
        if os.path.exists(f):
            return f
    return None


def _sources():
    return [os.path.join(CSRC, s) for s in SOURCES]


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "qfvm_gb300.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    ptxc = ptx_compiler_lib()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            extra = ["-DQSV_PTXCOMPILER"] if ptxc and os.path.basename(src) == "jit.cu" else []
            cmd = [cc] + ARCH + common + extra + ["-lineinfo", "-c", src, "-o", obj]
        else:
            cmd = [cc] + common + ["-x", "c++", "-c", src, "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 8))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ([ptxc, "-lpthread", "-lm"] if ptxc else []) + ["-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
