"""The C-ABI library loads and exports every symbol its header declares."""
import ctypes as C
import os
import re

import pytest

import jadamilu_gb300 as J

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="jadamilu_gb300.h", macro="JDG_API"):
    text = open(os.path.join(ROOT, "include", header)).read()
    return re.findall(macro + r"\s+[\w\s\*]+?\b(\w+)\s*\(", text)


def test_header_declares_the_drop_in_drivers():
    syms = set(declared_symbols())
    for s in ["dpjd_", "dpjdrevcom_", "djdrevcom_", "dpjd_gep_", "dpjdrevcom_gep_", "djdrevcom_gep_", "dpjdcleanup_",
              "zpjd_", "zpjdrevcom_", "zjdrevcom_", "zpjd_gep_", "zpjdrevcom_gep_", "zjdrevcom_gep_", "zpjdcleanup_"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    L = J.load()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_ilp64_library_exports_every_declared_symbol():
    from jadamilu_gb300 import build
    build.build_gpu()
    syms = declared_symbols("jadamilu_gb300_ilp64.h", "JDG64_API")
    assert len(syms) == 32  # 18 double / complex-double and legacy drivers, 14 single-precision
    L = C.CDLL(build.LIB64)
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_build_targets_sm103a_only():
    from jadamilu_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.exists(J.LIB_PATH)


def test_python_mirror_fails_loudly_without_gpu():
    L = J.load()
    if L.jdgpu_device_count() > 0:
        pytest.skip("a GPU is visible")
    from jadamilu_gb300 import matrices as M
    with pytest.raises(RuntimeError):
        J.dpjd(M.tridiag(50)[::-1], 3)
