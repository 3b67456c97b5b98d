"""End-to-end parity of the GPU drivers (through the C ABI) with the oracle.

Eigenvalues must agree with the oracle and the reference's printed values
within 1e-10 relative (absolute 1e-12 for the O(1) user-guide samples), and
residual norms must meet TOL.
"""
import numpy as np
import pytest

from jadamilu_gb300 import matrices as M
from problems import dense_eigs, kat_problem

pytestmark = pytest.mark.gpu


def _close(a, b, rel=1e-10, floor=1e-12):
    a, b = np.sort(a), np.sort(b)
    assert a.shape == b.shape
    assert np.all(np.abs(a - b) <= np.maximum(rel * np.abs(b), floor)), (a, b)


@pytest.mark.parametrize("name", ["EXAMPLE1", "EXAMPLE2", "EXAMPLE5", "EXAMPLE6", "EXAMPLE9", "EXAMPLE10"])
def test_userguide_samples(gpu, oracle, kats, name):
    meta = kats[name]
    A, As, mv, kw = kat_problem(meta)
    if meta["driver"] == "dpjd":
        r = gpu.dpjd((A[2], A[1], A[0]), 5, **kw)
        ro = oracle.dpjd(*A, 5, **kw)
    elif meta["driver"] == "dpjdrevcom":
        r = gpu.dpjdrevcom((A[2], A[1], A[0]), 5, mv, **kw)
        ro = oracle.dpjd(*A, 5, user_matvec=mv, **kw)
    else:
        d = As.diagonal().copy()
        neg = np.full(len(d) + 1, -1, np.int32)
        r = gpu.dpjdrevcom((d, neg, neg), 5, mv, **kw)
        ro = oracle.dpjd(neg, neg, d, 5, user_matvec=mv, **kw)
    assert r["info"] == 0 and r["neig"] == 5
    np.testing.assert_allclose(r["eigs"], meta["eigenvalues"], rtol=0, atol=1e-12)
    _close(r["eigs"], ro["eigs"])
    assert np.all(r["res"] <= 1e-10)
    # eigenvectors: unit norm, residual checked independently
    for k in range(5):
        x = r["x"][:, k]
        assert abs(np.linalg.norm(x) - 1) < 1e-10
        assert np.linalg.norm(mv(x) - r["eigs"][k] * x) < 1e-9


def test_laplace_20_cubed_plain_fp64(gpu, oracle):
    """Laplacian 20^3 (n=8000), 10 smallest, TOL 1e-10, DROPTOL 1e-3, FP64."""
    ia, ja, a = M.laplace3d(20)
    kw = dict(isearch=0, madspace=20, maxit=2000, tol=1e-10, droptol=1e-3, mem=20.0)
    r = gpu.dpjd((a, ja, ia), 10, **kw)
    assert r["info"] == 0 and r["neig"] == 10
    exact = M.laplace3d_eigenvalues(20, 10)
    _close(r["eigs"], exact)
    assert np.all(r["res"] <= 1e-10)
    ro = oracle.dpjd(ia, ja, a, 10, **kw)
    _close(r["eigs"], ro["eigs"])


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_anderson_interior(gpu, oracle, precision):
    ia, ja, a = M.anderson3d(12, seed=7)
    As = M.to_scipy_full(ia, ja, a)
    kw = dict(isearch=2, sigma=0.0, madspace=25, maxit=4000, tol=1e-10, droptol=1e-3, mem=40.0,
              icntl=(0, 1, 0, 0, precision))
    r = gpu.dpjd((a, ja, ia), 8, **kw)
    assert r["info"] == 0 and r["neig"] == 8
    _close(r["eigs"], dense_eigs(As, 8, 0.0))
    # convergence is declared on the inner solver's residual estimate (as in
    # the reference); the recomputed true residual may exceed TOL marginally
    # with the bfloat16 preconditioner
    assert np.all(r["res"] <= (1e-10 if precision < 2 else 2e-10))
    if precision < 2:
        ro = oracle.dpjd(ia, ja, a, 8, **kw)
        _close(r["eigs"], ro["eigs"])


def test_complex_hermitian(gpu, oracle):
    ia, ja, a = M.tight_binding3d(8, seed=1)
    As = M.to_scipy_full(ia, ja, a)
    kw = dict(isearch=0, madspace=20, maxit=2000, tol=1e-10, droptol=1e-3, icntl=(0, 1, 0, 0, 1))
    r = gpu.zpjd((a, ja, ia), 6, **kw)
    assert r["info"] == 0 and r["neig"] == 6
    _close(r["eigs"], dense_eigs(As, 6))
    ro = oracle.dpjd(ia, ja, a, 6, complex_=True, **kw)
    _close(r["eigs"], ro["eigs"])


def test_generalized(gpu, oracle):
    import scipy.linalg as sl
    K, Mm = M.fem_p1(16, seed=3)
    kw = dict(isearch=0, madspace=16, maxit=2000, tol=1e-9, droptol=1e-3)
    r = gpu.dpjd_gep((K[2], K[1], K[0]), (Mm[2], Mm[1], Mm[0]), 4, **kw)
    assert r["info"] == 0 and r["neig"] == 4
    w = sl.eigh(M.to_scipy_full(*K).toarray(), M.to_scipy_full(*Mm).toarray(), eigvals_only=True)[:4]
    _close(r["eigs"], w, rel=1e-9)
    ro = oracle.dpjd(*K, 4, b=Mm, **kw)
    _close(r["eigs"], ro["eigs"], rel=1e-9)


def test_djdrevcom_user_preconditioner(gpu):
    """DJDREVCOM with a user matvec and user preconditioner (EXAMPLE8 style)."""
    n = 1000
    import scipy.sparse as sp
    main = 4 * np.ones(n)
    A = sp.diags([main, -np.ones(n - 1), -np.ones(n - 1)], [0, -1, 1]).tolil()
    A[0, n - 1] = A[n - 1, 0] = -1
    A = A.tocsr()
    # the banded approximate inverse of samples/EXAMPLE8.f:73-87 (circulant)
    def prec(y):
        return (16 * y + 4 * (np.roll(y, 1) + np.roll(y, -1)) + (np.roll(y, 2) + np.roll(y, -2))) / 64.0
    r = gpu.djdrevcom(n, 5, lambda x: A @ x, prec, isearch=0, madspace=20, maxit=4000, tol=1e-10)
    assert r["info"] == 0 and r["neig"] == 5
    w = np.linalg.eigvalsh(A.toarray())[:5]
    _close(r["eigs"], w)


@pytest.mark.parametrize("case,info", [("neig", -5), ("madspace", -9), ("iter", -11), ("tol", -12)])
def test_info_codes(gpu, case, info):
    kw = dict(isearch=0, madspace=10, maxit=100, tol=1e-8)
    neig = 3
    if case == "neig":
        neig = 0
    elif case == "madspace":
        kw["madspace"] = 2
    elif case == "iter":
        kw["maxit"] = 0
    elif case == "tol":
        kw["tol"] = 0.0
    ia, ja, a = M.tridiag(60)
    r = gpu.dpjd((a, ja, ia), neig, **kw)
    assert r["info"] == info


def test_maxit_returns_partial(gpu):
    ia, ja, a = M.laplace3d(8)
    r = gpu.dpjd((a, ja, ia), 10, isearch=0, madspace=10, maxit=25, tol=1e-12, droptol=1e-1)
    assert r["info"] > 0


def test_legacy_pjd_forces_float64_preconditioner(gpu, kats):
    """PJD (src/jd/PJD_compatible.f:3-38) runs DPJD with ICNTL(5) = 0 and
    leaves the caller's ICNTL(5) as it was."""
    meta = kats["EXAMPLE1"]
    A, As, mv, kw = kat_problem(meta)
    kw = dict(kw, icntl=(0, 0, 0, 0, 1))
    r_leg = gpu.dpjd((A[2].copy(), A[1].copy(), A[0].copy()), 5, legacy=True, **kw)
    r_f64 = gpu.dpjd((A[2].copy(), A[1].copy(), A[0].copy()), 5, **dict(kw, icntl=(0, 0, 0, 0, 0)))
    assert r_leg["info"] == 0 and r_leg["neig"] == 5
    assert r_leg["icntl"][4] == 1
    np.testing.assert_array_equal(r_leg["eigs"], r_f64["eigs"])
    assert r_leg["iter"] == r_f64["iter"]
    np.testing.assert_allclose(r_leg["eigs"], meta["eigenvalues"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_dense_blocks_every_real_storage(gpu, precision):
    """Shallow test factors normally stay on the level path; with the dense
    blocks forced, the float64, float32 and bfloat16 tile kernels solve the
    Anderson 14^3 problem to the dense solver's eigenvalues."""
    ia, ja, a = M.anderson3d(14, seed=6)
    kw = dict(isearch=2, sigma=0.0, madspace=20, maxit=20000, tol=1e-10, droptol=1e-3, icntl=(0, 0, 0, 0, precision))
    gpu.set_option("dense_min_saving", -1.0)
    try:
        r = gpu.dpjd((a, ja, ia), 4, **kw)
        st = gpu.stats()
    finally:
        gpu.set_option("dense_min_saving", 1e-4)
    assert r["info"] == 0 and r["neig"] == 4
    assert st["dense_blocks"] >= 1 and st["dense_rows"] > 0
    w = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a).toarray())
    for lam in r["eigs"]:
        assert np.min(np.abs(w - lam)) <= 1e-9 * max(1.0, abs(lam))
    assert np.all(r["res"] <= (1e-10 if precision < 2 else 2e-10))


@pytest.mark.parametrize("precision", [0, 1])
def test_dense_blocks_complex_storage(gpu, precision):
    """The complex128 and complex64 tile kernels (forced dense blocks) on a
    complex Hermitian tight-binding problem, against the dense solver."""
    ia, ja, a = M.tight_binding3d(10, seed=3)
    kw = dict(isearch=0, sigma=0.0, madspace=20, maxit=20000, tol=1e-10, droptol=1e-3, icntl=(0, 0, 0, 0, precision))
    gpu.set_option("dense_min_saving", -1.0)
    try:
        r = gpu.zpjd((a, ja, ia), 4, **kw)
        st = gpu.stats(complex_=True)
    finally:
        gpu.set_option("dense_min_saving", 1e-4)
    assert r["info"] == 0 and r["neig"] == 4
    assert st["dense_blocks"] >= 1 and st["dense_rows"] > 0
    w = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a).toarray())
    np.testing.assert_allclose(np.sort(r["eigs"]), w[:4], rtol=1e-9, atol=1e-12)


def test_generalized_harmonic_interior(gpu, oracle):
    """DPJD_GEP with ISEARCH = 2 on the GPU: the eigenvalues of K x = lambda M x
    closest to an interior target, as the dense solver and the oracle give."""
    import scipy.linalg as sl
    K, Mm = M.fem_p1(24, seed=3)
    w = sl.eigh(M.to_scipy_full(*K).toarray(), M.to_scipy_full(*Mm).toarray(), eigvals_only=True)
    sigma = 0.5 * (w[7] + w[8])
    ref = np.sort(w[np.argsort(np.abs(w - sigma))[:5]])
    kw = dict(isearch=2, sigma=sigma, madspace=20, maxit=4000, tol=1e-9, droptol=1e-3)
    r = gpu.dpjd_gep((K[2], K[1], K[0]), (Mm[2], Mm[1], Mm[0]), 5, **kw)
    assert r["info"] == 0 and r["neig"] == 5
    np.testing.assert_allclose(np.sort(r["eigs"]), ref, rtol=1e-10)
    ro = oracle.dpjd(*K, 5, b=Mm, **kw)
    np.testing.assert_allclose(np.sort(r["eigs"]), np.sort(ro["eigs"]), rtol=1e-10)


def test_generalized_harmonic_complex(gpu):
    """ZPJD_GEP with ISEARCH = 2: complex Hermitian A, diagonal positive B."""
    import scipy.linalg as sl
    ia, ja, a = M.tight_binding3d(8, seed=4)
    n = len(ia) - 1
    bdiag = 1.0 + 0.5 * np.random.default_rng(9).uniform(size=n)
    ib = np.arange(1, n + 2, dtype=np.int32)
    jb = np.arange(1, n + 1, dtype=np.int32)
    b = bdiag.astype(np.complex128)
    Ad = M.to_scipy_full(ia, ja, a).toarray()
    w = sl.eigh(Ad, np.diag(bdiag), eigvals_only=True)
    sigma = 0.5 * (w[n // 2] + w[n // 2 + 1])
    ref = np.sort(w[np.argsort(np.abs(w - sigma))[:4]])
    r = gpu.zpjd_gep((a, ja, ia), (b, jb, ib), 4, isearch=2, sigma=sigma, madspace=20, maxit=6000, tol=1e-9,
                     droptol=1e-3)
    assert r["info"] == 0 and r["neig"] == 4
    np.testing.assert_allclose(np.sort(r["eigs"]), ref, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("coupling", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_anderson_large_form(gpu, oracle, coupling, precision):
    """Anderson 28^3 (n = 21952) with the factor form of 4096 rows and more,
    one global L (coupling 0) or per-level coupling blocks (coupling 1).  Ten
    interior eigenvalues against shift-and-invert Lanczos and the oracle (same
    factor form), residuals at TOL."""
    import ctypes as C
    from problems import shift_invert_eigs
    lib = oracle.lib()
    lib.orc_set_coupling.argtypes = [C.c_int]
    ia, ja, a = M.anderson3d(28, seed=0)
    kw = dict(isearch=2, sigma=0.0, madspace=25, maxit=20000, tol=1e-10, droptol=3e-3, mem=60.0,
              icntl=(0, 1, 0, 0, precision))
    lib.orc_set_coupling(coupling)
    gpu.set_option("coupling", coupling)
    try:
        r = gpu.dpjd((a, ja, ia), 10, **kw)
        ro = oracle.dpjd(ia, ja, a, 10, **kw)
    finally:
        lib.orc_set_coupling(0)
        gpu.set_option("coupling", 0)
    assert r["info"] == 0 and r["neig"] == 10
    As = M.to_scipy_full(ia, ja, a)
    _close(r["eigs"], shift_invert_eigs(As, 10))
    assert np.all(r["res"] <= 1.1e-10)
    _close(r["eigs"], ro["eigs"])


@pytest.mark.parametrize("m", [40, 60])
def test_anderson_bench_sizes_match_fixtures(gpu, m):
    """The benchmark's Anderson workload at 40^3 and 60^3 (seed 0, ten
    eigenpairs closest to 0, TOL 1e-10, float32 factor) against the committed
    fixtures (tests/golden/make_anderson_fixtures.py): shift-and-invert
    Lanczos (40^3) and the oracle.  Every returned eigenvalue equals one of
    the 14 eigenvalues closest to 0 within max(1e-10 |lambda|, 64 eps ||A||),
    ||A|| <= 6 + 8.25, and at least 9 of the 10 closest are returned: Jacobi-
    Davidson (the reference's too) can skip one member of a tight cluster and
    converge to the next eigenvalue instead.  Residuals at TOL."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "anderson_eigs.json")) as f:
        fx = json.load(f)
    case = fx["cases"][str(m)]
    ia, ja, a = M.anderson3d(m, disorder=16.5, seed=0)
    st = fx["settings"]
    r = gpu.dpjd((a, ja, ia), 10, isearch=st["isearch"], sigma=st["sigma"], madspace=st["madspace"],
                 maxit=st["maxit"], tol=st["tol"], droptol=st["droptol"], mem=st["mem"], icntl=tuple(st["icntl"]))
    assert r["info"] == 0 and r["neig"] == 10
    assert np.all(r["res"] <= 1.1e-10)
    floor = 64 * np.finfo(float).eps * (6 + 8.25)
    wide = np.array(case.get("shift_invert14", case.get("oracle14")))
    closest = wide[np.argsort(np.abs(wide), kind="stable")[:10]]
    for lam in r["eigs"]:
        assert np.min(np.abs(wide - lam)) <= max(1e-10 * abs(lam), floor), (lam, wide)
    found = sum(np.min(np.abs(r["eigs"] - w)) <= max(1e-10 * abs(w), floor) for w in closest)
    assert found >= 9, (np.sort(r["eigs"]), closest)


@pytest.mark.parametrize("m", [32, 64])
def test_tightbinding_matches_fixtures(gpu, m):
    """Complex Hermitian tight-binding workload (Peierls phases, phi = 1/17),
    8 smallest eigenvalues, complex128 outer / complex64 factor, at 32^3 and
    at the benchmark's 64^3 (n = 262,144), against the committed fixtures
    (tests/golden/make_tightbinding_fixtures.py): the oracle at both sizes and
    ARPACK Lanczos at 32^3.  Tolerance max(1e-10 |lambda|, 64 eps ||A||),
    ||A|| <= 6 + 2; residuals at TOL."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "tightbinding_eigs.json")) as f:
        fx = json.load(f)
    case = fx["cases"][str(m)]
    st = fx["settings"]
    ia, ja, a = M.tight_binding3d(m, phi=1.0 / 17.0, disorder=4.0, seed=1)
    r = gpu.zpjd((a, ja, ia), 8, isearch=st["isearch"], sigma=st["sigma"], madspace=st["madspace"],
                 maxit=st["maxit"], tol=st["tol"], droptol=st["droptol"], mem=st["mem"], icntl=tuple(st["icntl"]))
    assert r["info"] == 0 and r["neig"] == 8
    floor = 64 * np.finfo(float).eps * 8.0
    for key in ("lanczos", "oracle"):
        if key in case:
            _close(r["eigs"], np.array(case[key]), rel=1e-10, floor=floor)
    assert np.all(r["res"] <= 1.1e-10)


@pytest.mark.parametrize("m", [128, 512])
def test_fem_matches_fixtures(gpu, m):
    """Generalized FEM workload K x = lambda M x (P1, lognormal conductivity,
    lumped mass), 6 smallest eigenvalues, float64, at 128^2 nodes and at the
    benchmark's 512^2 (n = 260,100), against the committed fixtures
    (tests/golden/make_fem_fixtures.py): the oracle and ARPACK
    shift-and-invert at both sizes.  Tolerance max(1e-10 |lambda|, 64 eps
    lambda_max) with lambda_max the sixth eigenvalue."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "fem_eigs.json")) as f:
        fx = json.load(f)
    case = fx["cases"][str(m)]
    st = fx["settings"]
    K, Mm = M.fem_p1(m, sigma=0.5, seed=3)
    r = gpu.dpjd_gep((K[2], K[1], K[0]), (Mm[2], Mm[1], Mm[0]), 6, isearch=st["isearch"], sigma=st["sigma"],
                     madspace=st["madspace"], maxit=st["maxit"], tol=st["tol"], droptol=st["droptol"], mem=st["mem"],
                     icntl=tuple(st["icntl"]))
    assert r["info"] == 0 and r["neig"] == 6
    floor = 64 * np.finfo(float).eps * max(case["oracle"])
    for key in ("shift_invert", "oracle"):
        _close(r["eigs"], np.array(case[key]), rel=1e-10, floor=floor)


def test_anderson_100_cubed_headline(gpu):
    """The benchmark's headline workload at full size: Anderson 100^3
    (n = 1e6), ten eigenpairs closest to 0, fp32 factor, DROPTOL 1e-3.  The
    eigenvalues equal the oracle's complete solve (committed fixture) within
    max(1e-10 |lambda|, 64 eps ||A||), and every returned pair's residual
    ||A x - lambda x|| / ||x||, recomputed here in float64 by scipy, is at
    most 1.2 TOL."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "anderson_eigs.json")) as f:
        fx = json.load(f)
    st = fx["settings"]
    ia, ja, a = M.anderson3d(100, disorder=16.5, seed=0)
    r = gpu.dpjd((a, ja, ia), 10, isearch=st["isearch"], sigma=st["sigma"], madspace=st["madspace"],
                 maxit=st["maxit"], tol=st["tol"], droptol=st["droptol"], mem=st["mem"], icntl=tuple(st["icntl"]))
    assert r["info"] == 0 and r["neig"] == 10
    _close(r["eigs"], np.array(fx["cases"]["100"]["oracle"]), rel=1e-10, floor=64 * np.finfo(float).eps * 14.25)
    As = M.to_scipy_full(ia, ja, a).tocsr()
    X = r["x"]
    for k in range(10):
        x = X[:, k]
        res = np.linalg.norm(As @ x - r["eigs"][k] * x) / np.linalg.norm(x)
        assert res <= 1.2 * st["tol"], (k, res)
