"""Shared problem definitions for the oracle and GPU tests."""
import numpy as np

from jadamilu_gb300 import matrices as M


def kat_problem(meta):
    """(A, matvec, driver kwargs) for a user-guide sample (see golden/)."""
    ia, ja, a = M.tridiag(1000, diag_offset=meta["diag_offset"], diag_scale=meta["diag_scale"])
    As = M.to_scipy_full(ia, ja, a)
    kw = dict(isearch=meta["isearch"], sigma=meta.get("sigma", 0.0), madspace=20, maxit=1000, tol=1e-10,
              droptol=1e-3, mem=20.0, icntl=(meta.get("icntl1", 0), meta.get("icntl2", 0), 0, 0, 0))
    rank1 = meta.get("rank1")
    if rank1:
        mv = lambda x: As @ x + rank1 * x.sum()
    else:
        mv = lambda x: As @ x
    return (ia, ja, a), As, mv, kw


def dense_eigs(As, k, sigma=None):
    w = np.linalg.eigvalsh(As.toarray())
    if sigma is None:
        return w[:k]
    idx = np.argsort(np.abs(w - sigma), kind="stable")[:k]
    return np.sort(w[idx])


def shift_invert_eigs(As, k, sigma=0.0):
    """The k eigenvalues closest to sigma by shift-and-invert Lanczos (scipy's
    ARPACK on a sparse LU of As - sigma I): an independent check for matrices
    too large for a dense eigensolver."""
    import scipy.sparse.linalg as sla
    w = sla.eigsh(As.tocsc(), k=k, sigma=sigma, which="LM", tol=1e-13, return_eigenvectors=False)
    return np.sort(w)
