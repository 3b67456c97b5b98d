"""Sample drivers of the reference without printed outputs, run on the CPU
oracle: ISEARCH = 1 (EXAMPLE3/4: smallest eigenvalues with SHIFT as a lower
estimate) against the printed EXAMPLE2 eigenvalues of the same matrix and,
for the generalized problem, against scipy; the EXAMPLE7 pattern (a sequence
of nearby matrices solved with ICNTL(2) = -2, the previous preconditioner
kept, and NINIT initial vectors from the previous solve) against dense
solves; complex Hermitian interior eigenvalues against a dense solver."""
import json
import os

import numpy as np

from jadamilu_gb300 import matrices as M

HERE = os.path.dirname(os.path.abspath(__file__))


def test_isearch1_finds_example2_eigenvalues(oracle):
    meta = json.load(open(os.path.join(HERE, "golden", "userguide_kats.json")))["EXAMPLE2"]
    ia, ja, a = M.tridiag(1000, diag_offset=meta["diag_offset"], diag_scale=meta["diag_scale"])
    r = oracle.dpjd(ia, ja, a, 5, isearch=1, sigma=0.0, shift=-7.2, madspace=20, maxit=1000, tol=1e-10,
                    droptol=1e-3, mem=20.0)
    assert r["info"] == 0 and r["neig"] == 5
    np.testing.assert_allclose(np.sort(r["eigs"]), np.sort(meta["eigenvalues"]), rtol=0, atol=1e-10)
    assert np.all(r["res"] <= 1e-10)


def test_sequence_with_kept_preconditioner_and_initial_vectors(oracle):
    ia, ja, a = M.tridiag(1000, diag_offset=-1.0, diag_scale=1.0)
    kw = dict(isearch=0, sigma=0.0, madspace=20, maxit=2000, tol=1e-10, droptol=1e-3, mem=20.0)
    r1 = oracle.dpjd(ia.copy(), ja.copy(), a.copy(), 5, icntl=(0, 0, 0, 0, 0), **kw)
    assert r1["info"] == 0 and r1["neig"] == 5
    # the next matrix of the sequence: a small diagonal change
    rng = np.random.default_rng(3)
    a2 = a.copy()
    diag_pos = ia[:-1] - 1  # each row's first entry is its diagonal in this generator
    assert np.all(ja[diag_pos] - 1 == np.arange(len(ia) - 1))
    a2[diag_pos] += 1e-3 * rng.standard_normal(len(ia) - 1)
    w2 = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a2).toarray())[:5]
    order = np.argsort(r1["eigs"])
    x0 = r1["x"][:, order]
    warm = oracle.dpjd(ia.copy(), ja.copy(), a2.copy(), 5, ninit=5, x=x0, eigs=r1["eigs"][order],
                       icntl=(0, -2, 0, 0, 0), **kw)
    assert warm["info"] == 0 and warm["neig"] == 5
    np.testing.assert_allclose(np.sort(warm["eigs"]), w2, rtol=0, atol=1e-9)
    cold = oracle.dpjd(ia.copy(), ja.copy(), a2.copy(), 5, icntl=(0, 0, 0, 0, 0), **kw)
    assert cold["info"] == 0
    assert warm["iter"] < cold["iter"]


def test_generalized_isearch1_with_shift_estimate(oracle):
    """GEP with ISEARCH = 1: the smallest eigenvalues of K x = lambda M x, with
    SHIFT a lower estimate of them, against scipy."""
    import scipy.linalg as sl
    K, Mm = M.fem_p1(12, seed=3)
    Kd = M.to_scipy_full(*K).toarray()
    Md = M.to_scipy_full(*Mm).toarray()
    w = sl.eigh(Kd, Md, eigvals_only=True)
    r = oracle.dpjd(*K, 4, isearch=1, shift=0.5 * w[0], madspace=16, tol=1e-9, droptol=1e-3, b=Mm)
    assert r["info"] == 0 and r["neig"] == 4
    np.testing.assert_allclose(np.sort(r["eigs"]), w[:4], rtol=1e-9)


def test_complex_hermitian_isearch2_interior(oracle):
    """Complex Hermitian, eigenvalues closest to an interior target, against
    a dense solver."""
    ia, ja, a = M.tight_binding3d(6)
    As = M.to_scipy_full(ia, ja, a).toarray()
    w = np.linalg.eigvalsh(As)
    sigma = float(np.median(w))
    r = oracle.dpjd(ia, ja, a, 4, isearch=2, sigma=sigma, madspace=20, maxit=5000, tol=1e-10, droptol=1e-3,
                    complex_=True)
    assert r["info"] == 0 and r["neig"] == 4
    for lam in r["eigs"]:
        assert np.min(np.abs(w - lam)) <= 1e-9 * max(1.0, abs(lam))
    # the four closest to sigma, as JD with harmonic Ritz values reports them here
    ref = np.sort(w[np.argsort(np.abs(w - sigma))[:4]])
    np.testing.assert_allclose(np.sort(r["eigs"]), ref, rtol=0, atol=1e-9)
