"""The factor's maximum-product matching scale (csrc/matching.hpp, the role
of the reference's MC64 step, src/ilupack/symilupackfactor.c:184-193) against
brute force on small symmetric matrices: every scaled entry has modulus at
most 1, and the optimal matching's scaled product is exactly 1."""
import ctypes as C
import itertools

import numpy as np
import pytest

import oracle_lib as O


def _scale(A):
    L = O.lib()
    f = L.orc_matching_scale
    f.argtypes = [C.c_int] + [C.c_void_p] * 4
    f.restype = C.c_int
    n = A.shape[0]
    rp = np.zeros(n + 1, np.int32)
    ci, av = [], []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        ci += nz.tolist()
        av += A[i, nz].tolist()
        rp[i + 1] = len(ci)
    ci = np.array(ci, np.int32)
    av = np.array(av, np.float64)
    s = np.zeros(n)
    nm = f(n, rp.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p), av.ctypes.data_as(C.c_void_p),
           s.ctypes.data_as(C.c_void_p))
    return nm, s


@pytest.mark.parametrize("seed", range(40))
def test_matching_scale_is_optimal(seed):
    rng = np.random.default_rng(seed)
    n = 2 + seed % 6
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            if rng.random() < (0.5 if i == j else 0.6):
                A[i, j] = A[j, i] = np.exp(6 * (rng.random() - 0.5)) * (1 if rng.random() < 0.5 else -1)
    best = 0.0
    for p in itertools.permutations(range(n)):
        best = max(best, float(np.prod(np.abs(A[np.arange(n), p]))))
    nm, s = _scale(A)
    if best == 0.0:
        return  # structurally singular: no perfect matching to check
    assert nm == n
    S = np.abs(A) * np.outer(s, s)
    assert S.max() <= 1 + 1e-12
    assert abs(best * np.prod(s) ** 2 - 1.0) <= 1e-10


def test_matching_option_keeps_factor_exact():
    """With nothing dropped, the factor under the matching scale is still an
    exact LDL^T: its application solves the system."""
    from jadamilu_gb300 import matrices as M
    L = O.lib()
    ia, ja, a = M.anderson3d(6, seed=3)
    n = len(ia) - 1
    L.orc_set_matching(1)
    try:
        F = O.Factor(ia, ja, a, droptol=0.0, condest=1e30, mem=0.0)
        b = np.random.default_rng(0).standard_normal(n)
        x = F.apply(b)
    finally:
        L.orc_set_matching(0)
    A = M.to_scipy_full(ia, ja, a)
    assert np.linalg.norm(A @ x - b) <= 1e-9 * np.linalg.norm(b)
