"""Builds the in-tree shared libraries.

* ``jadamilu_gb300/_lib/libjadamilu_gb300.so``: the GPU library (nvcc,
  sm_103a only), translation units compiled in parallel;
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
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr",
           "-I" + os.path.join(ROOT, "include")]
UNITS = ["kernels.cu", "devjd.cu", "driver.cu", "grad.cu"]


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _sources():
    src = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".hpp", ".h"))]
    src.append(os.path.join(ROOT, "include", "jadamilu_gb300.h"))
    return src


def build_gpu(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(_sources()):
        return LIB
    nvcc = _nvcc()
    objs = []

    def comp(u):
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVFLAGS, "-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(comp, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
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
