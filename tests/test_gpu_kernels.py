"""Kernel parity: GPU SpMV and GPU preconditioner application vs the oracle."""
import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("gen", [lambda: M.laplace3d(12), lambda: M.anderson3d(15, seed=1),
                                 lambda: M.tridiag(1000), lambda: M.fem_p1(40)[0]])
def test_spmv_real(gpu, oracle, gen):
    ia, ja, a = gen()
    n = len(ia) - 1
    x = np.random.default_rng(0).standard_normal(n)
    y = gpu.spmv((a, ja, ia), x)
    yo = np.zeros(n)
    import ctypes as C
    p = lambda v: v.ctypes.data_as(C.c_void_p)
    oracle.lib().orc_dmatveca(n, p(ia), p(ja), p(a), p(x), p(yo))
    np.testing.assert_allclose(y, yo, rtol=1e-13, atol=1e-13 * np.abs(yo).max())


def test_spmv_complex(gpu, oracle):
    import ctypes as C
    ia, ja, a = M.tight_binding3d(10, seed=1)
    n = len(ia) - 1
    rng = np.random.default_rng(0)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = gpu.spmv((a, ja, ia), x)
    yo = np.zeros(n, np.complex128)
    p = lambda v: v.ctypes.data_as(C.c_void_p)
    oracle.lib().orc_zmatveca(n, p(ia), p(ja), p(a), p(x), p(yo))
    np.testing.assert_allclose(y, yo, rtol=1e-13, atol=1e-13 * np.abs(yo).max())


@pytest.mark.parametrize("spd", [False, True])
@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-5)])
@pytest.mark.parametrize("gen,shift", [(lambda: M.anderson3d(12, seed=2), 0.0), (lambda: M.laplace3d(12), 10.0),
                                       (lambda: M.tridiag(2000), 0.0)])
def test_ildl_apply_matches_oracle(gpu, oracle, gen, shift, spd, precision, tol):
    ia, ja, a = gen()
    n = len(ia) - 1
    F = oracle.Factor(ia, ja, a, shift=shift, droptol=1e-3, mem=0)
    assert F.ierr == 0
    B = np.random.default_rng(3).standard_normal((2, n))
    Xg, info = gpu.ildl_apply((a, ja, ia), B, shift=shift, droptol=1e-3, spd=spd, precision=precision)
    fi = F.info()
    assert info["nnz_l"] == fi["nnz_l"] and info["fwd_depth"] == fi["fwd_depth"]
    for r in range(2):
        xo = F.apply(B[r], spd=spd, single=(precision == 1))
        err = np.linalg.norm(Xg[r] - xo) / np.linalg.norm(xo)
        assert err <= tol, err


def test_ildl_apply_bf16_is_a_preconditioner(gpu, oracle):
    ia, ja, a = M.laplace3d(12)
    n = len(ia) - 1
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3, mem=0)
    b = np.random.default_rng(3).standard_normal(n)
    xb, _ = gpu.ildl_apply((a, ja, ia), b, shift=0.0, spd=True, precision=2)
    xo = F.apply(b, spd=True)
    assert np.linalg.norm(xb - xo) / np.linalg.norm(xo) < 5e-2


@pytest.mark.parametrize("variant", ["levels", "small_dense", "dense", "dense_cluster16"])
@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-5)])
def test_ildl_apply_tail_variants_match_oracle(gpu, oracle, variant, precision, tol):
    """The deepest levels solved level by level in one CTA, with the explicit
    inverse of a block capped at 100 rows, and with the block the cost model
    picks (tile products in clusters of 8 CTAs, or of 16 where the device
    allows) give the oracle's substitution result."""
    ia, ja, a = M.anderson3d(20, seed=3)
    n = len(ia) - 1
    F = oracle.Factor(ia, ja, a, shift=0.0, droptol=1e-3, mem=0)
    B = np.random.default_rng(4).standard_normal((2, n))
    try:
        if variant == "levels":
            gpu.set_option("dense_tail", 0)
        elif variant == "small_dense":
            gpu.set_option("dense_max", 100)
        elif variant == "dense_cluster16":
            gpu.set_option("tri_cluster", 16)
        Xg, info = gpu.ildl_apply((a, ja, ia), B, shift=0.0, droptol=1e-3, spd=False, precision=precision)
    finally:
        gpu.set_option("dense_tail", 1)
        gpu.set_option("dense_max", 32768)
        gpu.set_option("tri_cluster", 8)
    for r in range(2):
        # fp32 results are compared with the exact (fp64) application, within a
        # small multiple of the oracle's own fp32 substitution error
        xo = F.apply(B[r])
        err = np.linalg.norm(Xg[r] - xo) / np.linalg.norm(xo)
        if precision == 1:
            e32 = np.linalg.norm(F.apply(B[r], single=True) - xo) / np.linalg.norm(xo)
            tol = max(tol, 4 * e32)
        assert err <= tol, err


@pytest.mark.parametrize("coupling", [0, 1])
@pytest.mark.parametrize("spd", [False, True])
@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-5)])
def test_ildl_apply_large_form_matches_oracle(gpu, oracle, coupling, spd, precision, tol):
    """From 4096 rows on the factor defers pivots by look-ahead, drops by
    Schur contribution and factors its last level exactly; it keeps one global
    L (coupling 0, default) or each level's L and D apart with coupling blocks
    F (coupling 1, the multilevel form of symAMGsol.c:173-330, applied on the
    GPU as per-level sub-factors, F and F^H).  Anderson 28^3 (n = 21952)
    against the oracle's application of the same factor."""
    import ctypes as C
    lib = oracle.lib()
    lib.orc_set_coupling.argtypes = [C.c_int]
    ia, ja, a = M.anderson3d(28, seed=2)
    n = len(ia) - 1
    lib.orc_set_coupling(coupling)
    gpu.set_option("coupling", coupling)
    try:
        F = oracle.Factor(ia, ja, a, shift=0.0, droptol=3e-3, mem=0)
        assert F.ierr == 0 and F.info()["nlevels"] >= 2
        B = np.random.default_rng(5).standard_normal((2, n))
        Xg, info = gpu.ildl_apply((a, ja, ia), B, shift=0.0, droptol=3e-3, spd=spd, precision=precision)
    finally:
        lib.orc_set_coupling(0)
        gpu.set_option("coupling", 0)
    assert info["nnz_l"] == F.info()["nnz_l"]
    for r in range(2):
        xo = F.apply(B[r], spd=spd)
        err = np.linalg.norm(Xg[r] - xo) / np.linalg.norm(xo)
        if precision == 1:
            e32 = np.linalg.norm(F.apply(B[r], spd=spd, single=True) - xo) / np.linalg.norm(xo)
            tol = max(tol, 4 * e32)
        assert err <= tol, err
