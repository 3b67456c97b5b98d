"""The small dense solvers that stand in for LAPACK in SOLPROJEP and SHRINK
(src/jd/JDaux.F:3271-3358, 2418-2462; csrc/small_dense.hpp, shared by the
oracle and the GPU driver), against numpy / scipy on random matrices: the
Jacobi HEEV, HEGV (type 1), POSV, the complex-QR GEEV used by the harmonic
GEP extraction, and the Householder Q of the restart."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O

P = C.c_void_p


def _lib():
    L = O.lib()
    L.orc_heev.argtypes = [C.c_int, C.c_int, P, P]
    L.orc_hegv.argtypes = [C.c_int, C.c_int, P, P, P]
    L.orc_posv.argtypes = [C.c_int, C.c_int, P, P]
    L.orc_geev.argtypes = [C.c_int, P, P, P]
    L.orc_householder_q.argtypes = [C.c_int, C.c_int, P, P]
    return L


def _p(a):
    return a.ctypes.data_as(P)


def _herm(rng, J, cplx):
    X = rng.standard_normal((J, J)) + (1j * rng.standard_normal((J, J)) if cplx else 0)
    return (X + X.conj().T) / 2


@pytest.mark.parametrize("J", [1, 2, 5, 17, 32])
@pytest.mark.parametrize("cplx", [False, True])
def test_heev(J, cplx):
    rng = np.random.default_rng(J + 100 * cplx)
    A = _herm(rng, J, cplx)
    a = np.asfortranarray(A.astype(np.complex128 if cplx else np.float64))
    w = np.zeros(J)
    assert _lib().orc_heev(int(cplx), J, _p(a), _p(w)) == 0
    np.testing.assert_allclose(w, np.linalg.eigvalsh(A), rtol=0, atol=1e-13 * max(1, np.abs(A).max()) * J)
    V = a
    np.testing.assert_allclose(V.conj().T @ V, np.eye(J), atol=1e-13 * J)
    np.testing.assert_allclose(A @ V, V * w, atol=1e-12 * J)


@pytest.mark.parametrize("J", [1, 3, 12, 25])
@pytest.mark.parametrize("cplx", [False, True])
def test_hegv_and_posv(J, cplx):
    import scipy.linalg as sl
    rng = np.random.default_rng(7 * J + cplx)
    A = _herm(rng, J, cplx)
    G = rng.standard_normal((J, J)) + (1j * rng.standard_normal((J, J)) if cplx else 0)
    B = G @ G.conj().T + J * np.eye(J)
    dt = np.complex128 if cplx else np.float64
    a, b = np.asfortranarray(A.astype(dt)), np.asfortranarray(B.astype(dt))
    w = np.zeros(J)
    assert _lib().orc_hegv(int(cplx), J, _p(a), _p(b), _p(w)) == 0
    np.testing.assert_allclose(w, sl.eigh(A, B, eigvals_only=True), rtol=1e-12, atol=1e-12)
    Y = a
    np.testing.assert_allclose(Y.conj().T @ B @ Y, np.eye(J), atol=1e-11)
    # POSV: N X = M
    M = rng.standard_normal((J, J)) + (1j * rng.standard_normal((J, J)) if cplx else 0)
    n_, m_ = np.asfortranarray(B.astype(dt)), np.asfortranarray(M.astype(dt))
    assert _lib().orc_posv(int(cplx), J, _p(n_), _p(m_)) == 0
    np.testing.assert_allclose(m_, np.linalg.solve(B, M), rtol=1e-11, atol=1e-12)


def test_posv_reports_an_indefinite_matrix():
    N = np.asfortranarray(np.diag([2.0, -1.0, 3.0]))
    M = np.asfortranarray(np.eye(3))
    assert _lib().orc_posv(0, 3, _p(N), _p(M)) == 2


@pytest.mark.parametrize("J", [1, 2, 6, 20, 32])
def test_geev_real_spectrum_pencil(J):
    """B^{-1} A with A symmetric and B SPD has a real spectrum: eigenvalues
    against scipy, each eigenvector unit-norm with an exact eigen-residual."""
    import scipy.linalg as sl
    rng = np.random.default_rng(J)
    A = _herm(rng, J, False)
    G = rng.standard_normal((J, J))
    B = G @ G.T + J * np.eye(J)
    Mx = np.linalg.solve(B, A)
    a = np.asfortranarray(Mx)
    wr, V = np.zeros(J), np.asfortranarray(np.zeros((J, J)))
    assert _lib().orc_geev(J, _p(a), _p(wr), _p(V)) == 0
    np.testing.assert_allclose(np.sort(wr), np.sort(sl.eigvals(A, B).real), rtol=1e-10, atol=1e-12)
    for k in range(J):
        v = V[:, k]
        assert abs(np.linalg.norm(v) - 1) <= 1e-12
        assert np.linalg.norm(Mx @ v - wr[k] * v) <= 1e-9 * max(1, np.abs(Mx).max())


@pytest.mark.parametrize("K,J", [(5, 1), (8, 3), (32, 10)])
def test_householder_q_spans_u(K, J):
    rng = np.random.default_rng(K * J)
    U = np.asfortranarray(rng.standard_normal((K, J)))
    Q = np.zeros(K * K)
    _lib().orc_householder_q(K, J, _p(U), _p(Q))
    Q = Q.reshape(K, K, order="F")
    np.testing.assert_allclose(Q.T @ Q, np.eye(K), atol=1e-13)
    # the first J columns span U: the projection of U onto them is U
    Qj = Q[:, :J]
    np.testing.assert_allclose(Qj @ (Qj.T @ U), U, atol=1e-12)
