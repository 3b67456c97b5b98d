"""The host multilevel ILDLC factorisation (project code, no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from jadamilu_gb300 import matrices as M


def _random_indefinite(n, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=6.0 / n, random_state=seed)
    A = A + A.T + sp.diags(rng.uniform(-2, 2, n))
    U = sp.triu(A).tocsr()
    U.sort_indices()
    # diagonal must be present in every row
    U = (U + sp.diags(np.where(U.diagonal() == 0, 1e-3, 0.0))).tocsr()
    rows = np.repeat(np.arange(n), np.diff(U.indptr))
    return (U.indptr + 1).astype(np.int32), (U.indices + 1).astype(np.int32), U.data.astype(np.float64)


def _dense_indefinite(n, seed, density=0.4):
    """Symmetric indefinite matrix with 40 % of its entries set: the whole
    first level takes the dense elimination path."""
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=seed) * 0.1
    A = A + A.T + sp.diags(rng.uniform(-2, 2, n))
    U = sp.triu(A).tocsr()
    U = (U + sp.diags(np.where(U.diagonal() == 0, 1e-3, 0.0))).tocsr()
    U.sort_indices()
    return (U.indptr + 1).astype(np.int32), (U.indices + 1).astype(np.int32), U.data.astype(np.float64)


CASES = {
    "dense_indefinite": lambda: _dense_indefinite(500, 3),
    "laplace6": lambda: M.laplace3d(6),
    "anderson7": lambda: M.anderson3d(7, seed=2),
    "tridiag": lambda: M.tridiag(300),
    "tridiag_zero_diag": lambda: M.tridiag(300, diag_scale=0.0),
    "random_indefinite": lambda: _random_indefinite(400, 7),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_when_nothing_is_dropped(oracle, name):
    ia, ja, a = CASES[name]()
    A = M.to_scipy_full(ia, ja, a)
    import ctypes as C
    lib = oracle.lib()
    lib.orc_set_dense_min_rows.argtypes = [C.c_int]
    # small levels take the dense path here (by default only levels of 8192+ rows do)
    lib.orc_set_dense_min_rows(256 if name.startswith("dense") else -1)
    try:
        F = oracle.Factor(ia, ja, a, shift=0.1, droptol=0.0, mem=0)
    finally:
        lib.orc_set_dense_min_rows(-1)
    assert F.ierr == 0
    b = np.random.default_rng(1).standard_normal(A.shape[0])
    x = F.apply(b)
    As = A - 0.1 * sp.eye(A.shape[0])
    assert np.linalg.norm(As @ x - b) <= 1e-9 * np.linalg.norm(b) * max(1, np.abs(As).max())


def test_two_by_two_pivots_and_levels(oracle):
    ia, ja, a = M.anderson3d(8, seed=3)
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3)
    info = F.info()
    assert info["n2x2"] > 0          # indefinite: some 2x2 pivots
    assert info["nlevels"] >= 2      # deferred rows formed Schur levels
    assert info["nneg"] > 0


def test_spd_conversion_gives_spd_preconditioner(oracle):
    ia, ja, a = M.anderson3d(6, seed=4)
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3)
    n = F.n
    Mi = np.stack([F.apply(e, spd=True) for e in np.eye(n)], 1)
    np.testing.assert_allclose(Mi, Mi.T, atol=1e-10 * np.abs(Mi).max())
    assert np.linalg.eigvalsh(0.5 * (Mi + Mi.T)).min() > 0


def test_single_precision_apply_close(oracle):
    ia, ja, a = M.anderson3d(8, seed=3)
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3)
    b = np.random.default_rng(0).standard_normal(F.n)
    x64 = F.apply(b)
    x32 = F.apply(b, single=True)
    assert np.linalg.norm(x32 - x64) <= 1e-4 * np.linalg.norm(x64)


def test_memory_limit_reports_error(oracle):
    ia, ja, a = M.anderson3d(8, seed=3)
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=0.0, mem=1.5)
    assert F.ierr == -3


class _CoupledForm:
    """The coupling-block form (option coupling 1, from 4096 rows on) on
    small matrices: every level keeps its own L and D, the coupling blocks F
    are the level's matrix entries, the last level is exact once a third full."""

    def __init__(self, oracle):
        import ctypes as C
        self.lib = oracle.lib()
        self.lib.orc_set_coupled_min_n.argtypes = [C.c_int]
        self.lib.orc_set_coupling.argtypes = [C.c_int]

    def __enter__(self):
        self.lib.orc_set_coupled_min_n(0)
        self.lib.orc_set_coupling(1)
        return self

    def __exit__(self, *exc):
        self.lib.orc_set_coupled_min_n(4096)
        self.lib.orc_set_coupling(0)


@pytest.mark.parametrize("name", ["laplace6", "anderson7", "random_indefinite", "tridiag_zero_diag"])
def test_coupled_form_exact_when_nothing_is_dropped(oracle, name):
    ia, ja, a = CASES[name]()
    A = M.to_scipy_full(ia, ja, a)
    with _CoupledForm(oracle):
        F = oracle.Factor(ia, ja, a, shift=0.1, droptol=0.0, mem=0)
    assert F.ierr == 0
    b = np.random.default_rng(1).standard_normal(A.shape[0])
    x = F.apply(b)
    As = A - 0.1 * sp.eye(A.shape[0])
    assert np.linalg.norm(As @ x - b) <= 1e-9 * np.linalg.norm(b) * max(1, np.abs(As).max())


def test_coupled_form_levels_and_spd(oracle):
    """Deferred rows form levels; L has no entry across levels; the |D| form
    is Hermitian positive definite."""
    import ctypes as C
    ia, ja, a = M.anderson3d(7, seed=4)
    with _CoupledForm(oracle):
        F = oracle.Factor(ia, ja, a, shift=0.0, droptol=3e-3, mem=0)
    info = F.info()
    assert info["nlevels"] >= 2
    n = F.n
    L = oracle.lib()
    sizes = np.zeros(4, np.int64)
    L.orc_dfactor_schedule.argtypes = [C.c_void_p] * 8
    L.orc_dfactor_schedule(F.h, sizes.ctypes.data, None, None, None, None, None, None)
    nf, nb = int(sizes[0]), int(sizes[1])
    bufs = [np.zeros(nf + 1, np.int32), np.zeros(n, np.int32), np.zeros(nb + 1, np.int32), np.zeros(n, np.int32),
            np.zeros(n + 1, np.int64), np.zeros(int(sizes[3]), np.int32)]
    L.orc_dfactor_schedule(F.h, sizes.ctypes.data, *[v.ctypes.data for v in bufs])
    lp, li = bufs[4], bufs[5]
    flev = np.zeros(n, np.int32)
    ls = np.zeros(info["nlevels"] + 1, np.int32)
    L.orc_dfactor_levels.argtypes = [C.c_void_p] * 3
    L.orc_dfactor_levels(F.h, flev.ctypes.data, ls.ctypes.data)
    level_of = np.searchsorted(ls, np.arange(n), side="right") - 1
    rows = np.repeat(np.arange(n), np.diff(lp))
    assert np.array_equal(level_of[rows], level_of[li])
    Mi = np.stack([F.apply(e, spd=True) for e in np.eye(n)], 1)
    np.testing.assert_allclose(Mi, Mi.T, atol=1e-10 * np.abs(Mi).max())
    assert np.linalg.eigvalsh(0.5 * (Mi + Mi.T)).min() > 0


@pytest.mark.parametrize("large_form", [False, True])
def test_apply_matches_scipy_triangular_solves(oracle, large_form):
    """The oracle's application x = P (L D L^H)^{-1} P^T b checked against
    scipy: the factor's arrays (permutation, unit lower L, D^{-1} with 1x1
    and 2x2 blocks) exported and applied with scipy's sparse triangular
    solves, on an indefinite Anderson matrix with dropping (2x2 pivots,
    several levels), plain and large-matrix factor forms."""
    import ctypes as C
    from scipy.sparse.linalg import spsolve_triangular
    lib = oracle.lib()
    p = C.c_void_p
    lib.orc_set_coupled_min_n.argtypes = [C.c_int]
    lib.orc_set_coupled_min_n(0 if large_form else 1 << 30)
    try:
        ia, ja, a = M.anderson3d(10, seed=5)
        F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3)
    finally:
        lib.orc_set_coupled_min_n(4096)
    assert F.ierr == 0
    sizes = np.zeros(4, np.int64)
    lib.orc_dfactor_schedule.argtypes = [p] * 8
    lib.orc_dfactor_schedule(F.h, sizes.ctypes.data, None, None, None, None, None, None)
    n, nz = int(sizes[2]), int(sizes[3])
    perm, lp, li = np.zeros(n, np.int32), np.zeros(n + 1, np.int64), np.zeros(nz, np.int32)
    lx, blk, dinv, doff = np.zeros(nz), np.zeros(n, np.int8), np.zeros(n), np.zeros(n)
    lib.orc_dfactor_export.argtypes = [p] * 8
    lib.orc_dfactor_export(F.h, *[v.ctypes.data for v in (perm, lp, li, lx, blk, dinv, doff)])
    assert F.info()["n2x2"] > 0 and F.info()["nlevels"] >= 2
    L = sp.csr_matrix((lx, li, lp), shape=(n, n)) + sp.eye(n, format="csr")
    Dinv = sp.lil_matrix((n, n))
    for s in range(n):
        if blk[s] == 1:
            Dinv[s, s] = dinv[s]
        elif blk[s] == 2:
            Dinv[s, s], Dinv[s + 1, s + 1] = dinv[s], dinv[s + 1]
            Dinv[s, s + 1] = Dinv[s + 1, s] = doff[s]
    b = np.random.default_rng(3).standard_normal(n)
    y = spsolve_triangular(L.tocsr(), b[perm], lower=True, unit_diagonal=True)
    y = Dinv.tocsr() @ y
    y = spsolve_triangular(L.T.tocsr(), y, lower=False, unit_diagonal=True)
    x_ref = np.empty(n)
    x_ref[perm] = y
    x = F.apply(b)
    assert np.linalg.norm(x - x_ref) <= 1e-12 * np.linalg.norm(x_ref)
