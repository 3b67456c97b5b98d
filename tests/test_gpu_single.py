"""Single-precision drivers (SPJD / CPJD families, reference
Doc/SPJD_prototypes.f and Doc/CPJD_prototypes.f): REAL / COMPLEX arguments
in front of the double GPU drivers.  The direct drivers give exactly the
rounded results of the double drivers on the rounded inputs; the reverse-
communication drivers serve single-precision user operators."""
import ctypes as C

import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

pytestmark = pytest.mark.gpu
P = C.c_void_p


def _p(a):
    return a.ctypes.data_as(P)


def _i(v):
    return np.array([v], np.int32)


def _lx(n, neig, mad, gep=False):
    return n * ((4 if gep else 3) * mad + neig + 4) + 3 * mad * mad + max(mad * mad, neig)


def _direct(L, name, n, a, ja, ia, neig, rdt, vdt, kw, B=None):
    mad = kw["madspace"]
    lx = _lx(n, neig, mad, B is not None)
    A = np.array(a, vdt)
    JA, IA = np.array(ja, np.int32), np.array(ia, np.int32)
    X = np.zeros(lx, vdt)
    EIGS, RES = np.zeros(neig, rdt), np.zeros(neig, rdt)
    sc = {k: np.array([kw[k]], rdt) for k in ("sigma", "tol", "shift", "droptol", "mem")}
    GAP = np.zeros(1, rdt)
    N, LX, NEIG, ISEARCH, NINIT, MAD, ITER = (_i(v) for v in (n, lx, neig, kw["isearch"], 0, mad, kw["maxit"]))
    ICNTL, IPRINT, INFO = np.zeros(5, np.int32), _i(0), _i(0)
    args = [_p(N), _p(A), _p(JA), _p(IA)]
    if B is not None:
        Bv, JB, IB = np.array(B[0], vdt), np.array(B[1], np.int32), np.array(B[2], np.int32)
        args += [_p(Bv), _p(JB), _p(IB)]
    args += [_p(EIGS), _p(RES), _p(X), _p(LX), _p(NEIG), _p(sc["sigma"]), _p(ISEARCH), _p(NINIT), _p(MAD), _p(ITER),
             _p(sc["tol"]), _p(sc["shift"]), _p(sc["droptol"]), _p(sc["mem"]), _p(ICNTL), _p(IPRINT), _p(INFO),
             _p(GAP)]
    f = getattr(L, name)
    f.argtypes = [P] * len(args)
    f(*args)
    k = int(NEIG[0])
    return int(INFO[0]), EIGS[:k].copy(), int(ITER[0]), X[:n * k].reshape(k, n).T.copy()


KW = dict(sigma=0.0, isearch=2, madspace=20, maxit=5000, tol=1e-7, shift=0.0, droptol=1e-3, mem=20.0)


def test_spjd_is_rounded_dpjd(gpu):
    L = gpu.load()
    ia, ja, a = M.anderson3d(10, seed=5)
    n = len(ia) - 1
    a32 = np.asarray(a, np.float32)
    kw32 = {k: (float(np.float32(v)) if isinstance(v, float) else v) for k, v in KW.items()}
    info_s, eig_s, it_s, x_s = _direct(L, "spjd_", n, a32, ja, ia, 4, np.float32, np.float32, kw32)
    info_d, eig_d, it_d, x_d = _direct(L, "dpjd_", n, a32.astype(np.float64), ja, ia, 4, np.float64, np.float64, kw32)
    assert info_s == 0 and info_d == 0 and it_s == it_d
    assert np.array_equal(eig_s, eig_d.astype(np.float32))
    assert np.array_equal(x_s, x_d.astype(np.float32))
    w = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a32.astype(np.float64)).toarray())
    ref = np.sort(w[np.argsort(np.abs(w))[:4]])
    np.testing.assert_allclose(np.sort(eig_s), ref, rtol=1e-5, atol=1e-6)


def test_spjd_gep_is_rounded_dpjd_gep(gpu):
    L = gpu.load()
    K, Mm = M.fem_p1(12, seed=3)
    n = len(K[0]) - 1
    kw = dict(KW, isearch=0)
    k32 = np.asarray(K[2], np.float32)
    m32 = np.asarray(Mm[2], np.float32)
    info_s, eig_s, it_s, _ = _direct(L, "spjd_gep_", n, k32, K[1], K[0], 4, np.float32, np.float32, kw,
                                     B=(m32, Mm[1], Mm[0]))
    info_d, eig_d, it_d, _ = _direct(L, "dpjd_gep_", n, k32.astype(np.float64), K[1], K[0], 4, np.float64,
                                     np.float64, kw, B=(m32.astype(np.float64), Mm[1], Mm[0]))
    assert info_s == 0 and info_d == 0 and it_s == it_d
    assert np.array_equal(eig_s, eig_d.astype(np.float32))


def test_cpjd_is_rounded_zpjd(gpu):
    L = gpu.load()
    ia, ja, a = M.tight_binding3d(8)
    n = len(ia) - 1
    kw = dict(KW, isearch=0)
    a64 = np.asarray(a, np.complex64)
    info_c, eig_c, it_c, _ = _direct(L, "cpjd_", n, a64, ja, ia, 4, np.float32, np.complex64, kw)
    info_z, eig_z, it_z, _ = _direct(L, "zpjd_", n, a64.astype(np.complex128), ja, ia, 4, np.float64, np.complex128,
                                     kw)
    assert info_c == 0 and info_z == 0 and it_c == it_z
    assert np.array_equal(eig_c, eig_z.astype(np.float32))


def test_sjdrevcom_single_precision_operators(gpu):
    """SJDREVCOM with a float32 matvec and a float32 diagonal preconditioner:
    the eigenvalues of the float32-rounded matrix to single-precision
    accuracy, and the request vectors handed out in float32."""
    L = gpu.load()
    ia, ja, a = M.anderson3d(8, seed=7)
    n = len(ia) - 1
    As = M.to_scipy_full(ia, ja, np.asarray(a, np.float32).astype(np.float64)).astype(np.float32).tocsr()
    p = (np.abs(As.diagonal()) + 1).astype(np.float32)
    neig, mad = 4, 20
    lx = _lx(n, neig, mad)
    X = np.zeros(lx, np.float32)
    EIGS, RES, GAP = np.zeros(neig, np.float32), np.zeros(neig, np.float32), np.zeros(1, np.float32)
    SIGMA, TOL = np.array([0.0], np.float32), np.array([1e-5], np.float32)
    N, LX, NEIG, ISEARCH, NINIT, MAD, ITER = (_i(v) for v in (n, lx, neig, 0, 0, mad, 20000))
    IJOB, NDX1, NDX2, IPRINT, INFO = (_i(0) for _ in range(5))
    L.sjdrevcom_.argtypes = [P] * 18
    calls = 0
    while True:
        L.sjdrevcom_(_p(N), _p(EIGS), _p(RES), _p(X), _p(LX), _p(NEIG), _p(SIGMA), _p(ISEARCH), _p(NINIT), _p(MAD),
                     _p(ITER), _p(TOL), _p(IJOB), _p(NDX1), _p(NDX2), _p(IPRINT), _p(INFO), _p(GAP))
        job = int(IJOB[0])
        if job == 0:
            break
        i1, i2 = int(NDX1[0]) - 1, int(NDX2[0]) - 1
        if job == 1:
            X[i2:i2 + n] = As @ X[i1:i1 + n]
        else:
            X[i1:i1 + n] = X[i2:i2 + n] / p
        calls += 1
        assert calls < 200000
    assert INFO[0] == 0 and NEIG[0] == neig
    w = np.linalg.eigvalsh(As.toarray().astype(np.float64))
    for lam in EIGS:
        assert np.min(np.abs(w - lam)) <= 1e-4 * max(1.0, abs(lam))


def _spjdrevcom_diag(L, name, n, d, As, neig, rdt, kw):
    """SPJDREVCOM / DPJDREVCOM with JA(1) < 0: A holds the N diagonal values,
    JA and IA have one element each.  The user matvec runs in float32 for
    both: DPJDREVCOM's request vectors are rounded to float32 first, as the
    single-precision driver hands them out."""
    mad = kw["madspace"]
    lx = _lx(n, neig, mad)
    A = np.array(d, rdt)
    JA, IA = np.array([-1], np.int32), np.array([-7], np.int32)  # IA must not be read
    X = np.zeros(lx, rdt)
    EIGS, RES, GAP = np.zeros(neig, rdt), np.zeros(neig, rdt), np.zeros(1, rdt)
    sc = {k: np.array([kw[k]], rdt) for k in ("sigma", "tol", "shift", "droptol", "mem")}
    N, LX, NEIG, ISEARCH, NINIT, MAD, ITER = (_i(v) for v in (n, lx, neig, kw["isearch"], 0, mad, kw["maxit"]))
    ICNTL, IJOB, NDX1, NDX2, IPRINT, INFO = np.zeros(5, np.int32), _i(0), _i(0), _i(0), _i(0), _i(0)
    f = getattr(L, name)
    f.argtypes = [P] * 25
    Am = As.astype(np.float32)
    while True:
        f(_p(N), _p(A), _p(JA), _p(IA), _p(EIGS), _p(RES), _p(X), _p(LX), _p(NEIG), _p(sc["sigma"]), _p(ISEARCH),
          _p(NINIT), _p(MAD), _p(ITER), _p(sc["tol"]), _p(sc["shift"]), _p(sc["droptol"]), _p(sc["mem"]), _p(ICNTL),
          _p(IJOB), _p(NDX1), _p(NDX2), _p(IPRINT), _p(INFO), _p(GAP))
        if IJOB[0] == 0:
            break
        assert IJOB[0] == 1
        i1, i2 = int(NDX1[0]) - 1, int(NDX2[0]) - 1
        X[i2:i2 + n] = Am @ X[i1:i1 + n].astype(np.float32)
    k = int(NEIG[0])
    return int(INFO[0]), EIGS[:k].copy(), int(ITER[0]), A, JA, IA


def test_spjdrevcom_diagonal_preconditioning(gpu):
    """JA(1) < 0 (PJD.F:309-317): the single-precision revcom driver reads only
    A(1..N), never IA, leaves A/JA/IA unchanged, and returns the rounded
    results of DPJDREVCOM on the same rounded data."""
    L = gpu.load()
    ia, ja, a = M.anderson3d(8, seed=7)
    n = len(ia) - 1
    As = M.to_scipy_full(ia, ja, np.asarray(a, np.float32).astype(np.float64)).tocsr()
    d32 = As.diagonal().astype(np.float32)
    kw = dict(KW, isearch=0, maxit=20000)
    kw32 = {k: (float(np.float32(v)) if isinstance(v, float) else v) for k, v in kw.items()}
    info_s, eig_s, it_s, A_s, JA_s, IA_s = _spjdrevcom_diag(L, "spjdrevcom_", n, d32, As, 4, np.float32, kw32)
    assert info_s == 0 and len(eig_s) == 4
    assert np.array_equal(A_s, d32) and JA_s[0] == -1 and IA_s[0] == -7
    info_d, eig_d, it_d, A_d, _, _ = _spjdrevcom_diag(L, "dpjdrevcom_", n, d32.astype(np.float64), As, 4, np.float64,
                                                      kw32)
    assert info_d == 0 and it_s == it_d
    assert np.array_equal(eig_s, eig_d.astype(np.float32))
    w = np.linalg.eigvalsh(As.toarray())
    for lam in eig_s:
        assert np.min(np.abs(w - lam)) <= 1e-4 * max(1.0, abs(lam))
