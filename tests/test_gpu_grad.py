"""Gradients on the P1-FEM generalized problem K x = lambda M x: eigenvalue
gradients (jdgpu_deig_grad) against the Hellmann-Feynman formula evaluated in
numpy and against central finite differences of the eigenvalue sum (the
differentiation configuration's check, at a reduced grid); the gradient of an
eigenvector loss (jdgpu_deigvec_grad, adjoint MINRES on the GPU) against
central finite differences."""
import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

pytestmark = pytest.mark.gpu


def _rows_cols(ia, ja):
    n = len(ia) - 1
    return np.repeat(np.arange(n), np.diff(ia)), np.asarray(ja) - 1


def test_eig_grad_matches_formula_any_scaling(gpu):
    import scipy.linalg as sl
    K, Mm = M.fem_p1(20, seed=3)
    ia, ja, a = K
    Kd = M.to_scipy_full(*K).toarray()
    md = M.to_scipy_full(*Mm).toarray().diagonal()
    w, X = sl.eigh(Kd, np.diag(md))
    X = X[:, :6]
    rows, cols = _rows_cols(ia, ja)
    wts = np.array([1.0, 0.5, 2.0, 1.0, -1.0, 3.0])
    ref = np.sum(wts * X[rows] * X[cols], 1) * np.where(rows == cols, 1.0, 2.0)
    # the entry point normalises by x^T M x, so scaled eigenvectors give the same gradient
    scale = np.array([1.0, -3.0, 0.25, 7.0, 1e-3, 2.0])
    g = gpu.eig_grad((a, ja, ia), X * scale, w=wts, bdiag=md)
    np.testing.assert_allclose(g, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_eig_grad_of_gpu_eigenpairs_matches_central_differences(gpu):
    """Gradient of the sum of the 6 smallest eigenvalues from the GPU solver's
    eigenvectors, against central differences on 40 seeded stored entries.
    Step 1e-6 (the configuration's step): the differences carry rounding of
    about eps*|f|/h, so the bound is 1e-5 of max|g|; step 1e-4: 1e-6."""
    import scipy.linalg as sl
    K, Mm = M.fem_p1(20, seed=3)
    r = gpu.dpjd_gep((K[2], K[1], K[0]), (Mm[2], Mm[1], Mm[0]), 6, isearch=0, madspace=20, maxit=4000,
                     tol=1e-10, droptol=1e-3)
    assert r["info"] == 0 and r["neig"] == 6
    a, ja, ia = r["a"], r["ja"], r["ia"]
    md = M.to_scipy_full(*Mm).toarray().diagonal()
    g = gpu.eig_grad((a, ja, ia), r["x"][:, :6], bdiag=md)
    Kd = M.to_scipy_full(ia, ja, a).toarray()
    rows, cols = _rows_cols(ia, ja)
    qs = np.random.default_rng(7).choice(len(a), 40, replace=False)
    for h, bound in ((1e-6, 1e-5), (1e-4, 1e-6)):
        fd = np.empty(len(qs))
        for t, q in enumerate(qs):
            i, j = rows[q], cols[q]
            f = []
            for sgn in (1.0, -1.0):
                Kp = Kd.copy()
                Kp[i, j] += sgn * h
                if i != j:
                    Kp[j, i] += sgn * h
                f.append(np.sum(sl.eigh(Kp, np.diag(md), eigvals_only=True)[:6]))
            fd[t] = (f[0] - f[1]) / (2 * h)
        err = np.max(np.abs(fd - g[qs])) / np.max(np.abs(g))
        assert err <= bound, (h, err)


def test_eigvec_loss_grad_matches_central_differences(gpu):
    """Gradient of L(x) = c^T x for the third eigenvector of the FEM pencil
    (from the GPU solver), by the adjoint MINRES solve on the GPU, against
    central differences (step 1e-6) on 20 seeded stored entries of K."""
    import scipy.linalg as sl
    K, Mm = M.fem_p1(20, seed=3)
    md = M.to_scipy_full(*Mm).toarray().diagonal()
    r = gpu.dpjd_gep((K[2], K[1], K[0]), (Mm[2], Mm[1], Mm[0]), 3, isearch=0, madspace=20, maxit=4000,
                     tol=1e-11, droptol=1e-3)
    assert r["info"] == 0 and r["neig"] == 3
    a, ja, ia = r["a"], r["ja"], r["ia"]
    order = np.argsort(r["eigs"])
    lam, x = r["eigs"][order[2]], r["x"][:, order[2]].copy()
    x /= np.sqrt(x @ (md * x))
    n = len(ia) - 1
    c = np.random.default_rng(1).standard_normal(n)
    grad, its, res = gpu.eigvec_grad((a, ja, ia), lam, x, c, bdiag=md, tol=1e-12, maxit=3000)
    assert res <= 1e-10, (its, res)
    Kd = M.to_scipy_full(ia, ja, a).toarray()
    Bd = np.diag(md)
    rows = np.repeat(np.arange(n), np.diff(ia))
    cols = np.asarray(ja) - 1

    def loss(Kmat):
        w, X = sl.eigh(Kmat, Bd)
        xx = X[:, 2]
        return c @ (xx if xx @ (md * x) > 0 else -xx)

    h = 1e-6
    err = 0.0
    for q in np.random.default_rng(7).choice(len(a), 20, replace=False):
        i, j = rows[q], cols[q]
        f = []
        for sgn in (1.0, -1.0):
            Kp = Kd.copy()
            Kp[i, j] += sgn * h
            if i != j:
                Kp[j, i] += sgn * h
            f.append(loss(Kp))
        err = max(err, abs((f[0] - f[1]) / (2 * h) - grad[q]))
    assert err <= 1e-6 * np.abs(grad).max(), err


def test_eig_grad_fem512_central_differences(gpu, oracle):
    """The differentiation configuration at full size: P1-FEM K x = lambda M x
    on 512 x 512 nodes (n = 260,100), gradient of the sum of the 6 smallest
    eigenvalues with respect to every stored entry of K (jdgpu_deig_grad),
    against central differences with step h = 1e-6 on 100 seeded entries.
    Each difference re-solves K +- h E_q on the GPU (warm start from the
    unperturbed eigenvectors, the kept preconditioner: ICNTL(2) = -1).

    Bound: 1e-6 max|g| plus the rounding floor of a difference quotient,
    16 eps sum|lambda| / h (the eigenvalue sums carry rounding of a few eps
    |lambda| each).  For 3 of the entries the oracle (the reference's
    algorithm on the CPU) solves the same perturbed pencils: its eigenvalues
    agree with the GPU's to 1e-10 relative and its differences meet the same
    bound."""
    K, Mm = M.fem_p1(512, seed=3)
    B = (Mm[2], Mm[1], Mm[0])
    kw = dict(isearch=0, madspace=20, maxit=20000, tol=1e-10, droptol=1e-3)
    r = gpu.dpjd_gep((K[2], K[1], K[0]), B, 6, icntl=(0, 1, 0, 0, 0), **kw)
    assert r["info"] == 0 and r["neig"] == 6
    a, ja, ia = r["a"], r["ja"], r["ia"]  # DPJD put each row's diagonal first
    md = M.to_scipy_full(*Mm).diagonal()
    order = np.argsort(r["eigs"])
    X0 = r["x"][:, order].copy()
    g = gpu.eig_grad((a, ja, ia), X0, bdiag=md)
    h = 1e-6
    floor = 16 * np.finfo(float).eps * np.sum(np.abs(r["eigs"])) / h
    bound = 1e-6 * np.abs(g).max() + floor
    qs = np.random.default_rng(11).choice(len(a), 100, replace=False)
    sums = {}
    worst = 0.0
    for q in qs:
        f = []
        for sgn in (1.0, -1.0):
            ap = a.copy()
            ap[q] += sgn * h
            rp = gpu.dpjd_gep((ap, ja, ia), B, 6, ninit=6, x=X0, icntl=(0, -1, 0, 0, 0), **kw)
            assert rp["info"] == 0 and rp["neig"] == 6
            f.append(np.sort(rp["eigs"]))
        sums[int(q)] = f
        worst = max(worst, abs((f[0].sum() - f[1].sum()) / (2 * h) - g[q]))
    assert worst <= bound, (worst, bound)
    # the oracle at the same perturbed inputs (its own kept factor of K)
    ro = oracle.dpjd(ia, ja, a, 6, b=(Mm[0], Mm[1], Mm[2]), ninit=6, x=X0, icntl=(0, 1, 0, 0, 0), **kw)
    assert ro["info"] == 0
    for q in qs[:3]:
        fo = []
        for k, sgn in enumerate((1.0, -1.0)):
            ap = a.copy()
            ap[q] += sgn * h
            rp = oracle.dpjd(ia, ja, ap, 6, b=(Mm[0], Mm[1], Mm[2]), ninit=6, x=X0, icntl=(0, -1, 0, 0, 0), **kw)
            assert rp["info"] == 0 and rp["neig"] == 6
            eo = np.sort(rp["eigs"])
            np.testing.assert_allclose(eo, sums[int(q)][k], rtol=1e-10, atol=0)
            fo.append(eo.sum())
        assert abs((fo[0] - fo[1]) / (2 * h) - g[q]) <= bound
