"""The C-ABI library loads and exports every symbol its header declares."""
import ctypes as C
import os
import re

import pytest

import jadamilu_gb300 as J

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            out += re.findall(r"JDG_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return out


def test_header_declares_the_drop_in_drivers():
    syms = set(declared_symbols())
    for s in ["dpjd_", "dpjdrevcom_", "djdrevcom_", "dpjd_gep_", "dpjdrevcom_gep_", "djdrevcom_gep_", "dpjdcleanup_",
              "zpjd_", "zpjdrevcom_", "zjdrevcom_", "zpjd_gep_", "zpjdrevcom_gep_", "zjdrevcom_gep_", "zpjdcleanup_"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    L = J.load()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_library_is_sm103a_only():
    assert os.path.exists(J.LIB_PATH)
    data = open(J.LIB_PATH, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def test_python_mirror_fails_loudly_without_gpu():
    L = J.load()
    if L.jdgpu_device_count() > 0:
        pytest.skip("a GPU is visible")
    from jadamilu_gb300 import matrices as M
    with pytest.raises(RuntimeError):
        J.dpjd(M.tridiag(50)[::-1], 3)
