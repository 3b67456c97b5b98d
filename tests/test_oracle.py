"""The CPU oracle against the reference's printed results and exact spectra.

The reference has no test suite; the user guide's sample outputs
(Doc/userguide.ps, extracted into golden/userguide_kats.json) pin the
restatement, together with closed-form and dense eigenvalues.
"""
import numpy as np
import pytest

from jadamilu_gb300 import matrices as M
from problems import dense_eigs, kat_problem


@pytest.mark.parametrize("name", ["EXAMPLE1", "EXAMPLE2", "EXAMPLE5", "EXAMPLE6", "EXAMPLE9", "EXAMPLE10"])
def test_userguide_samples(oracle, kats, name):
    meta = kats[name]
    A, As, mv, kw = kat_problem(meta)
    if meta["driver"] == "dpjd":
        r = oracle.dpjd(*A, 5, **kw)
    elif meta["driver"] == "dpjdrevcom":
        r = oracle.dpjd(*A, 5, user_matvec=mv, **kw)
    else:  # diagonal preconditioning: JA(1) = IA(1) = -1, A holds the diagonal
        d = As.diagonal().copy()
        neg = np.full(len(d) + 1, -1, np.int32)  # only JA(1) < 0 matters; IA sets N here
        r = oracle.dpjd(neg, neg, d, 5, user_matvec=mv, **kw)
    assert r["info"] == 0
    assert r["neig"] == 5
    np.testing.assert_allclose(r["eigs"], meta["eigenvalues"], rtol=0, atol=1e-12)
    assert np.all(r["res"] <= 1e-10)
    if meta["driver"] == "dpjdrevcom_diag":
        # same preconditioner as the reference: the iteration itself matches
        # up to rounding-order effects (one step at most on these samples)
        assert abs(r["iter"] - meta["matvec"]) <= 1


def test_diag_example9_matvec_count_exact(oracle, kats):
    """EXAMPLE9 uses the reference's own diagonal preconditioner: 166 MATVECs."""
    meta = kats["EXAMPLE9"]
    A, As, mv, kw = kat_problem(meta)
    neg = np.full(As.shape[0] + 1, -1, np.int32)
    r = oracle.dpjd(neg, neg, As.diagonal().copy(), 5, user_matvec=mv, **kw)
    assert r["iter"] == meta["matvec"] == 166


def test_laplace_closed_form(oracle):
    m = 8
    ia, ja, a = M.laplace3d(m)
    r = oracle.dpjd(ia, ja, a, 10, isearch=0, madspace=20, tol=1e-10, droptol=1e-3)
    assert r["info"] == 0
    exact = M.laplace3d_eigenvalues(m, 10)
    np.testing.assert_allclose(r["eigs"], exact, rtol=1e-10)


def test_anderson_interior_dense(oracle):
    ia, ja, a = M.anderson3d(8, seed=5)
    As = M.to_scipy_full(ia, ja, a)
    r = oracle.dpjd(ia, ja, a, 6, isearch=2, sigma=0.0, madspace=20, tol=1e-10, droptol=1e-3)
    assert r["info"] == 0 and r["neig"] == 6
    np.testing.assert_allclose(np.sort(r["eigs"]), dense_eigs(As, 6, 0.0), rtol=0, atol=1e-10)


def test_anderson_interior_mixed(oracle):
    ia, ja, a = M.anderson3d(8, seed=5)
    As = M.to_scipy_full(ia, ja, a)
    r = oracle.dpjd(ia, ja, a, 6, isearch=2, sigma=0.0, madspace=20, tol=1e-10, droptol=1e-3,
                    icntl=(0, 0, 0, 0, 1))
    assert r["info"] == 0
    np.testing.assert_allclose(np.sort(r["eigs"]), dense_eigs(As, 6, 0.0), rtol=0, atol=1e-10)


def test_complex_hermitian(oracle):
    ia, ja, a = M.tight_binding3d(6, seed=1)
    As = M.to_scipy_full(ia, ja, a)
    r = oracle.dpjd(ia, ja, a, 4, isearch=0, madspace=16, tol=1e-10, droptol=1e-3, complex_=True)
    assert r["info"] == 0
    np.testing.assert_allclose(r["eigs"], dense_eigs(As, 4), rtol=0, atol=1e-10)


def test_generalized(oracle):
    import scipy.linalg as sl
    K, Mm = M.fem_p1(12, seed=3)
    Kd = M.to_scipy_full(*K).toarray()
    Md = M.to_scipy_full(*Mm).toarray()
    r = oracle.dpjd(*K, 4, isearch=0, madspace=16, tol=1e-9, droptol=1e-3, b=Mm)
    assert r["info"] == 0
    w = sl.eigh(Kd, Md, eigvals_only=True)[:4]
    np.testing.assert_allclose(r["eigs"], w, rtol=1e-9)


@pytest.mark.parametrize("case,info", [("n", -1), ("neig", -5), ("madspace", -9), ("lx", -10), ("iter", -11),
                                       ("tol", -12)])
def test_info_codes(oracle, case, info):
    import ctypes as C
    L = oracle.lib()
    ia, ja, a = M.tridiag(50)
    n, neig, mad, it, tol, lx = 50, 3, 10, 100, 1e-8, 10000
    if case == "n":
        n = 1
    elif case == "neig":
        neig = 0
    elif case == "madspace":
        mad = 2
    elif case == "lx":
        lx = 10
    elif case == "iter":
        it = 0
    elif case == "tol":
        tol = 0.0
    X = np.zeros(max(lx, 1))
    E = np.zeros(5)
    R = np.zeros(5)
    NEIG = np.array([neig], np.int32)
    ITER = np.array([it], np.int32)
    INFO = np.zeros(1, np.int32)
    GAP = np.zeros(1)
    p = lambda v: v.ctypes.data_as(C.c_void_p)
    L.orc_djd(n, p(E), p(R), p(X), lx, p(NEIG), 0.0, 0, 0, mad, p(ITER), tol, p(INFO), p(GAP), 0, None, None, None)
    assert INFO[0] == info


@pytest.mark.parametrize("m,neig", [(16, 4), (24, 5)])
def test_generalized_harmonic_interior(oracle, m, neig):
    """K x = lambda M x with ISEARCH = 2 (SOLPROJEP's POSV + GEEV branch):
    the eigenvalues closest to an interior target."""
    import scipy.linalg as sl
    K, Mm = M.fem_p1(m, seed=3)
    w = sl.eigh(M.to_scipy_full(*K).toarray(), M.to_scipy_full(*Mm).toarray(), eigvals_only=True)
    sigma = 0.5 * (w[7] + w[8])
    ref = np.sort(w[np.argsort(np.abs(w - sigma))[:neig]])
    r = oracle.dpjd(*K, neig, b=Mm, isearch=2, sigma=sigma, madspace=20, maxit=4000, tol=1e-9, droptol=1e-3)
    assert r["info"] == 0 and r["neig"] == neig
    np.testing.assert_allclose(np.sort(r["eigs"]), ref, rtol=1e-10)
