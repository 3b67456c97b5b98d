"""The explicit inverse of a dense block's unit lower-triangular part
(csrc/tail_inverse.hpp), which the GPU's tile product multiplies by: tiles of
L^{-1} (forward set) and L^{-H} (backward set), 64 x 64, column-major, packed
by tile rows; the work items that split each tile row over a thread-block
cluster.  Host code, checked on the CPU against numpy."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O

T = 64


def _tiles(m, L, threads):
    lib = O.lib()
    f = lib.orc_tail_inverse
    f.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    rp = [0]
    ci, cv = [], []
    for i in range(m):
        for j in range(i):
            if L[i, j] != 0:
                ci.append(j)
                cv.append(L[i, j])
        rp.append(len(ci))
    rp = np.array(rp, np.int64)
    ci = np.array(ci, np.int32)
    cv = np.array(cv, np.float64)
    nt = (m + T - 1) // T
    ntiles = nt * (nt + 1) // 2
    tf = np.full(ntiles * T * T, np.nan)
    tb = np.full(ntiles * T * T, np.nan)
    r = f(m, rp.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p), cv.ctypes.data_as(C.c_void_p), threads,
          tf.ctypes.data_as(C.c_void_p), tb.ctypes.data_as(C.c_void_p))
    assert r == nt
    return nt, tf.reshape(ntiles, T, T), tb.reshape(ntiles, T, T)


def _assemble(nt, tiles, lower):
    """Dense matrix from packed tiles (tile element (r, c) at c*64 + r)."""
    M = np.zeros((nt * T, nt * T))
    q = 0
    for i in range(nt):
        for j in (range(i + 1) if lower else range(i, nt)):
            M[i * T:(i + 1) * T, j * T:(j + 1) * T] = tiles[q].T  # stored column-major
            q += 1
    return M


@pytest.mark.parametrize("m,density,threads", [(1, 0.0, 1), (63, 0.3, 1), (64, 0.2, 2), (150, 0.05, 3),
                                               (200, 0.5, 4)])
def test_tiles_hold_the_inverse_and_its_adjoint(m, density, threads):
    rng = np.random.default_rng(m)
    L = np.tril(rng.standard_normal((m, m)) * (rng.random((m, m)) < density), -1) * 0.3 + np.eye(m)
    nt, tf, tb = _tiles(m, L, threads)
    Linv = np.linalg.inv(L)
    F = _assemble(nt, tf, True)
    B = _assemble(nt, tb, False)
    np.testing.assert_allclose(F[:m, :m], Linv, rtol=0, atol=1e-10 * np.abs(Linv).max())
    np.testing.assert_allclose(B[:m, :m], Linv.T, rtol=0, atol=1e-10 * np.abs(Linv).max())
    # entries past the block's order are zero
    assert np.all(F[m:, :] == 0) and np.all(F[:, m:] == 0) and np.all(B[m:, :] == 0)


def test_tiles_do_not_depend_on_the_thread_count():
    rng = np.random.default_rng(5)
    m = 300
    L = np.tril(rng.standard_normal((m, m)) * (rng.random((m, m)) < 0.1), -1) * 0.2 + np.eye(m)
    _, f1, b1 = _tiles(m, L, 1)
    _, f7, b7 = _tiles(m, L, 7)
    assert np.array_equal(f1, f7) and np.array_equal(b1, b7)


@pytest.mark.parametrize("nt,lower,per_row", [(1, True, 8), (5, True, 8), (5, False, 8), (87, True, 8),
                                              (20, False, 3)])
def test_cluster_items_cover_each_tile_row_once(nt, lower, per_row):
    lib = O.lib()
    f = lib.orc_cluster_items
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p]
    f.restype = C.c_int
    out = np.zeros(nt * per_row * 4, np.int32)
    k = f(nt, int(lower), per_row, out.ctypes.data_as(C.c_void_p))
    assert k == nt * per_row
    items = out.reshape(-1, 4)
    for i in range(nt):
        mine = items[i * per_row:(i + 1) * per_row]
        assert np.all(mine[:, 0] == i)  # the cluster of row i holds exactly its items, in rank order
        cols = []
        for row, first, cnt, c0 in mine:
            assert cnt >= 0
            cols += list(range(c0, c0 + cnt))
            # storage index of the first tile matches the packed layout
            off = i * (i + 1) // 2 if lower else i * nt - i * (i - 1) // 2
            base_col = 0 if lower else i
            if cnt:
                assert first == off + (c0 - base_col)
        want = list(range(0, i + 1)) if lower else list(range(i, nt))
        assert cols == want
