"""Builds the in-tree shared libraries.

* ``jadamilu_gb300/_lib/libjadamilu_gb300.so``: the GPU library (nvcc,
  sm_103a only), translation units compiled in parallel;
* ``jadamilu_gb300/_lib/libjadamilu_gb300_ilp64.so``: the same drivers with
  64-bit integer arguments (driver.cu compiled a second time with
  JDG_ILP64_INNER behind the wrappers of ilp64.cpp);
* ``oracle/_build/liboracle.so``: the CPU oracle used by the tests, the
  smoke check and the CPU-baseline leg of bench.py.

Rebuilds only what is older than its sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libjadamilu_gb300.so")
LIB64 = os.path.join(OUT, "libjadamilu_gb300_ilp64.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr",
           "-I" + os.path.join(ROOT, "include")]
UNITS = ["kernels.cu", "devjd.cu", "driver.cu", "grad.cu", "single.cpp"]
# (source, object, extra flags) of the ILP64 library's own units
UNITS64 = [("driver.cu", "driver_i32.o", ["-DJDG_ILP64_INNER"]), ("single.cpp", "single_i32.o", ["-DJDG_ILP64_INNER"]),
           ("ilp64.cpp", "ilp64.o", [])]


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _sources():
    src = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".hpp", ".h", ".cpp"))]
    src.append(os.path.join(ROOT, "include", "jadamilu_gb300.h"))
    src.append(os.path.join(ROOT, "include", "jadamilu_gb300_ilp64.h"))
    return src


def build_gpu(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    newest = _newest(_sources())
    if (not force and all(os.path.exists(p) and os.path.getmtime(p) >= newest for p in (LIB, LIB64))):
        return LIB
    nvcc = _nvcc()

    def comp(job):
        src, obj, extra = job
        obj = os.path.join(OUT, obj)
        cmd = [nvcc, *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    jobs = [(u, os.path.splitext(u)[0] + ".o", []) for u in UNITS] + UNITS64
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(comp, jobs))
    # the ILP64 library has its own drivers; the single-precision ones are 32-bit only
    common = [o for o in objs[: len(UNITS)] if not o.endswith(("driver.o", "single.o"))]
    for lib, parts in ((LIB, objs[: len(UNITS)]), (LIB64, common + objs[len(UNITS):])):
        tmp = lib + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *parts, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed for {os.path.basename(lib)}:\n{r.stderr[-4000:]}")
        os.replace(tmp, lib)
    return LIB


def build_oracle(force: bool = False) -> str:
    args = ["make", "-s", "-C", ORACLE_DIR]
    if force:
        args.append("-B")
    subprocess.check_call(args)
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gpu, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    import sys
    build_all(force="-f" in sys.argv)
    print(LIB)
