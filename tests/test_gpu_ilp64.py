"""The 64-bit-integer drivers (libjadamilu_gb300_ilp64.so, include/
jadamilu_gb300_ilp64.h) through ctypes with int64 arrays: DPJD on a user-guide
sample against its printed eigenvalues, and DPJDREVCOM with a user matvec
against a dense solver."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from jadamilu_gb300 import matrices as M
from problems import kat_problem

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
P = C.c_void_p


def _lib64():
    from jadamilu_gb300 import build
    build.build_gpu()
    return C.CDLL(build.LIB64)


def _i8(v):
    return np.array([v], np.int64)


def _p(a):
    return a.ctypes.data_as(P)


def test_ilp64_dpjd_userguide_sample(gpu):
    kats = json.load(open(os.path.join(HERE, "golden", "userguide_kats.json")))
    meta = kats["EXAMPLE1"]
    (ia, ja, a), As, mv, kw = kat_problem(meta)
    L = _lib64()
    n, neig, mad = len(ia) - 1, 5, kw["madspace"]
    ia8, ja8, a8 = np.asarray(ia, np.int64), np.asarray(ja, np.int64), np.array(a, np.float64)
    lx = n * (3 * mad + neig + 4) + 3 * mad * mad + max(mad * mad, neig)
    X = np.zeros(lx)
    EIGS, RES = np.zeros(neig), np.zeros(neig)
    N, LX, NEIG, ISEARCH, NINIT, MAD, ITER = (_i8(v) for v in (n, lx, neig, kw["isearch"], 0, mad, kw["maxit"]))
    ICNTL = np.array(kw["icntl"], np.int64)
    IPRINT, INFO = _i8(0), _i8(0)
    SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP = (np.array([v]) for v in (kw["sigma"], kw["tol"], 0.0, kw["droptol"],
                                                                      kw["mem"], 0.0))
    L.dpjd_.argtypes = [P] * 22
    L.dpjd_(_p(N), _p(a8), _p(ja8), _p(ia8), _p(EIGS), _p(RES), _p(X), _p(LX), _p(NEIG), _p(SIGMA), _p(ISEARCH),
            _p(NINIT), _p(MAD), _p(ITER), _p(TOL), _p(SHIFT), _p(DROPTOL), _p(MEM), _p(ICNTL), _p(IPRINT), _p(INFO),
            _p(GAP))
    assert INFO[0] == 0 and NEIG[0] == neig
    np.testing.assert_allclose(EIGS, meta["eigenvalues"], rtol=0, atol=1e-12)
    # the driver put each row's diagonal entry first, in JA too
    rows = np.repeat(np.arange(n), np.diff(ia8))
    first = ia8[:-1] - 1
    assert np.all(ja8[first] - 1 == rows[first])


def test_ilp64_dpjdrevcom_user_matvec(gpu):
    ia, ja, a = M.anderson3d(10, seed=5)
    As = M.to_scipy_full(ia, ja, a)
    L = _lib64()
    n, neig, mad = len(ia) - 1, 4, 20
    ia8, ja8, a8 = np.asarray(ia, np.int64), np.asarray(ja, np.int64), np.array(a, np.float64)
    lx = n * (3 * mad + neig + 4) + 3 * mad * mad + max(mad * mad, neig)
    X = np.zeros(lx)
    EIGS, RES = np.zeros(neig), np.zeros(neig)
    N, LX, NEIG, ISEARCH, NINIT, MAD, ITER = (_i8(v) for v in (n, lx, neig, 2, 0, mad, 5000))
    ICNTL = np.zeros(5, np.int64)
    IJOB, NDX1, NDX2, IPRINT, INFO = (_i8(0) for _ in range(5))
    SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP = (np.array([v]) for v in (0.0, 1e-10, 0.0, 1e-3, 20.0, 0.0))
    L.dpjdrevcom_.argtypes = [P] * 25
    calls = 0
    while True:
        L.dpjdrevcom_(_p(N), _p(a8), _p(ja8), _p(ia8), _p(EIGS), _p(RES), _p(X), _p(LX), _p(NEIG), _p(SIGMA),
                      _p(ISEARCH), _p(NINIT), _p(MAD), _p(ITER), _p(TOL), _p(SHIFT), _p(DROPTOL), _p(MEM), _p(ICNTL),
                      _p(IJOB), _p(NDX1), _p(NDX2), _p(IPRINT), _p(INFO), _p(GAP))
        if IJOB[0] != 1:
            break
        i1, i2 = NDX1[0] - 1, NDX2[0] - 1
        X[i2:i2 + n] = As @ X[i1:i1 + n]
        calls += 1
        assert calls < 100000
    assert INFO[0] == 0 and NEIG[0] == neig
    w = np.linalg.eigvalsh(As.toarray())
    ref = np.sort(w[np.argsort(np.abs(w))[:neig]])
    np.testing.assert_allclose(np.sort(EIGS), ref, rtol=1e-9, atol=1e-12)
