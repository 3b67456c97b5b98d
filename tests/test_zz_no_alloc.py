"""The allocation-free preconditioner entry point (jdgpu_dildl_apply_noalloc).

Some callers cannot call cudaMalloc, for instance an application whose GPU
memory all belongs to a framework's caching allocator, or one that fixes its
device-memory budget at start-up.  The entry point gives them the
preconditioner application of jdgpu_dildl_apply with every device buffer
carved out of a fixed array inside the library.  These tests call both entry
points through the C ABI and require the same results, on two calls in a row
(the shared array keeps the previous call's contents, which must not leak
into the next result), and check that an oversized problem is refused.

This file is collected last on purpose: a run that stops at the first
failure has then already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

pytestmark = pytest.mark.gpu

_P = C.c_void_p


def _apply(gpu, name, A, B, shift, spd, precision):
    L = gpu.load()
    f = getattr(L, name)
    f.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _P, _P, _P]
    f.restype = C.c_int
    ia, ja, a = (np.ascontiguousarray(A[0], np.int32), np.ascontiguousarray(A[1], np.int32),
                 np.ascontiguousarray(A[2], np.float64))
    n = len(ia) - 1
    B = np.ascontiguousarray(B, np.float64).reshape(-1, n)
    X = np.zeros_like(B)
    info = np.zeros(5, np.int64)
    p = lambda v: v.ctypes.data_as(_P)
    rc = f(n, p(ia), p(ja), p(a), shift, 1e-3, 5.0, int(spd), int(precision), B.shape[0], p(B), p(X), p(info))
    return rc, X, info


CASES = [
    # (matrix, shift, spd, precision, tolerance used by the kernel parity tests)
    (lambda: M.anderson3d(12, seed=2), 0.0, False, 0, 1e-11),
    (lambda: M.laplace3d(12), 10.0, True, 1, 2e-5),
]


def test_noalloc_matches_allocating_entry_on_consecutive_calls(gpu):
    rng = np.random.default_rng(11)
    for gen, shift, spd, precision, tol in CASES:  # two calls in a row, different problems
        A = gen()
        n = len(A[0]) - 1
        B = rng.standard_normal((2, n))
        rc0, X0, info0 = _apply(gpu, "jdgpu_dildl_apply", A, B, shift, spd, precision)
        rc1, X1, info1 = _apply(gpu, "jdgpu_dildl_apply_noalloc", A, B, shift, spd, precision)
        assert rc0 == 0 and rc1 == 0
        assert np.array_equal(info0, info1)
        for r in range(2):
            err = np.linalg.norm(X1[r] - X0[r]) / np.linalg.norm(X0[r])
            assert err <= tol, err


def test_noalloc_repeat_call_same_result(gpu):
    A = M.anderson3d(10, seed=4)
    n = len(A[0]) - 1
    B = np.random.default_rng(5).standard_normal((1, n))
    rc1, X1, _ = _apply(gpu, "jdgpu_dildl_apply_noalloc", A, B, 0.0, False, 0)
    rc2, X2, _ = _apply(gpu, "jdgpu_dildl_apply_noalloc", A, B, 0.0, False, 0)
    rc0, X0, _ = _apply(gpu, "jdgpu_dildl_apply", A, B, 0.0, False, 0)
    assert rc1 == rc2 == rc0 == 0
    assert np.linalg.norm(X2 - X0) <= 1e-11 * np.linalg.norm(X0)
    assert np.linalg.norm(X1 - X0) <= 1e-11 * np.linalg.norm(X0)


def test_noalloc_rejects_problems_beyond_the_scratch_size(gpu):
    A = M.tridiag(1_500_000)  # about 90 MB of device data, more than the 32 MiB array
    n = len(A[0]) - 1
    B = np.ones((1, n))
    rc, _, _ = _apply(gpu, "jdgpu_dildl_apply_noalloc", A, B, 0.0, False, 0)
    assert rc == -98
    # the library stays usable afterwards
    A2 = M.tridiag(200)
    rc2, X2, _ = _apply(gpu, "jdgpu_dildl_apply_noalloc", A2, np.ones((1, 200)), 0.0, False, 0)
    rc3, X3, _ = _apply(gpu, "jdgpu_dildl_apply", A2, np.ones((1, 200)), 0.0, False, 0)
    assert rc2 == 0 and rc3 == 0
    assert np.linalg.norm(X2 - X3) <= 1e-11 * np.linalg.norm(X3)
