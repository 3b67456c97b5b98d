"""The level schedules the GPU sweeps run (ildlc_levels in csrc/ildlc.hpp):
every row once; in the forward schedule every row's L entries point to rows
of earlier levels, with one in the level just before (levels as shallow as
possible); in the backward schedule the same holds for L^H."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from jadamilu_gb300 import matrices as M

P = C.c_void_p


def _schedule(F):
    L = O.lib()
    f = L.orc_dfactor_schedule
    f.argtypes = [P] * 8
    sizes = np.zeros(4, np.int64)
    f(F.h, sizes.ctypes.data_as(P), None, None, None, None, None, None)
    nf, nb, n, nnz = (int(v) for v in sizes)
    fptr, frows = np.zeros(nf + 1, np.int32), np.zeros(n, np.int32)
    bptr, brows = np.zeros(nb + 1, np.int32), np.zeros(n, np.int32)
    lp, li = np.zeros(n + 1, np.int64), np.zeros(max(nnz, 1), np.int32)
    f(F.h, sizes.ctypes.data_as(P), fptr.ctypes.data_as(P), frows.ctypes.data_as(P), bptr.ctypes.data_as(P),
      brows.ctypes.data_as(P), lp.ctypes.data_as(P), li.ctypes.data_as(P))
    return fptr, frows, bptr, brows, lp, li[:nnz]


def _check(ptr, rows, deps, n):
    assert sorted(rows.tolist()) == list(range(n))
    lev = np.empty(n, np.int64)
    for l in range(len(ptr) - 1):
        lev[rows[ptr[l]:ptr[l + 1]]] = l
    for r in range(n):
        d = deps[r]
        if len(d) == 0:
            assert lev[r] == 0
        else:
            assert lev[d].max() == lev[r] - 1


@pytest.mark.parametrize("m,droptol", [(6, 1e-3), (10, 3e-3), (12, 0.0)])
def test_schedules_respect_dependencies(m, droptol):
    ia, ja, a = M.anderson3d(m, seed=2)
    F = O.Factor(ia, ja, a, droptol=droptol, mem=0.0)
    fptr, frows, bptr, brows, lp, li = _schedule(F)
    n = F.n
    fdeps = [li[lp[r]:lp[r + 1]] for r in range(n)]  # row r of L needs columns li
    bd = [[] for _ in range(n)]  # row c of L^H needs the rows r with L(r, c) != 0
    for r in range(n):
        for c in fdeps[r]:
            bd[c].append(r)
    bdeps = [np.array(v, np.int64) for v in bd]
    _check(fptr, frows, fdeps, n)
    _check(bptr, brows, bdeps, n)
    assert len(fptr) - 1 == F.info()["fwd_depth"]
