"""The dense-block planner (csrc/block_plan.hpp): over random level
structures, the plan is contiguous from its first group to the last level,
respects the row cap, and attains the minimum of its cost model over every
way of cutting the levels (brute-force enumeration); shallow structures get
the empty plan."""
import ctypes as C
import itertools

import numpy as np
import pytest

import oracle_lib as O

T_LAUNCH, BW, TILE = 4e-6, 5.0e12, 64


def _plan(fptr, ef, eb, elem, dense_max, min_saving):
    L = O.lib()
    f = L.orc_plan_blocks
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
    f.restype = C.c_int
    nfl = len(fptr) - 1
    fp = np.array(fptr, np.int32)
    a, b = np.array(ef, np.int64), np.array(eb, np.int64)
    out = np.zeros(3 * nfl, np.int32)
    k = f(nfl, fp.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), elem,
          dense_max, min_saving, out.ctypes.data_as(C.c_void_p))
    return [tuple(out[3 * i:3 * i + 3]) for i in range(k)]


def _costs(fptr, ef, eb, elem):
    eb_ = elem + 4
    lev = [(2 if l > 0 else 1) * T_LAUNCH + (ef[l] + eb[l]) * eb_ / BW for l in range(len(fptr) - 1)]

    def dense(a, b):
        m = fptr[b] - fptr[a]
        nt = (m + TILE - 1) // TILE
        ent = sum(ef[l] + eb[l] for l in range(a, b))
        return 6 * T_LAUNCH + 2.0 * nt * (nt + 1) / 2 * TILE * TILE * elem / BW + ent * eb_ / BW
    return lev, dense


def _brute(fptr, ef, eb, elem, dense_max):
    """Minimum modelled cost over all cuts of levels 1..nfl-1 into single
    levels and dense blocks (level 0 always stays a level)."""
    nfl = len(fptr) - 1
    lev, dense = _costs(fptr, ef, eb, elem)
    best = np.inf
    for cuts in itertools.product([0, 1], repeat=max(0, nfl - 2)):
        bounds = [1] + [l for l, c in zip(range(2, nfl), cuts) if c] + [nfl]
        total = lev[0]
        ok = True
        for a, b in zip(bounds[:-1], bounds[1:]):
            opts = []
            if b - a == 1:
                opts.append(lev[a])
            if fptr[b] - fptr[a] <= dense_max:
                opts.append(dense(a, b))
            if not opts:
                ok = False
                break
            total += min(opts)
        if ok:
            best = min(best, total)
    return best


def _plan_cost(plan, fptr, ef, eb, elem):
    nfl = len(fptr) - 1
    lev, dense = _costs(fptr, ef, eb, elem)
    if not plan:
        return sum(lev)
    first = plan[0][0]
    total = sum(lev[:first])
    for a, b, d in plan:
        total += dense(a, b) if d else lev[a]
    return total


@pytest.mark.parametrize("seed", range(25))
def test_plan_is_optimal_for_its_model(seed):
    rng = np.random.default_rng(seed)
    nfl = int(rng.integers(3, 10))
    rows = rng.integers(1, 400, size=nfl)
    fptr = np.concatenate([[0], np.cumsum(rows)]).tolist()
    ef = (rows * rng.integers(1, 40, size=nfl)).tolist()
    eb = (rows * rng.integers(0, 40, size=nfl)).tolist()
    elem = int(rng.choice([2, 4, 8]))
    dense_max = int(rng.choice([300, 800, 100000]))
    plan = _plan(fptr, ef, eb, elem, dense_max, 0.0)
    if plan:
        assert plan[-1][1] == nfl and plan[0][0] >= 1
        for (a, b, d), nxt in zip(plan, plan[1:] + [None]):
            assert b > a and (d or b == a + 1)
            assert not d or fptr[b] - fptr[a] <= dense_max
            if nxt is not None:
                assert nxt[0] == b
    best = _brute(fptr, ef, eb, elem, dense_max)
    got = _plan_cost(plan, fptr, ef, eb, elem)
    assert got <= best * (1 + 1e-12) + 1e-18


def test_shallow_structure_keeps_the_level_path():
    fptr = [0, 10, 20, 30]
    ef, eb = [10, 20, 30], [10, 20, 30]
    assert _plan(fptr, ef, eb, 4, 32768, 100e-6) == []


def test_deep_chain_gets_dense_blocks():
    """Many one-row levels (a long dependency chain) cost one launch each; a
    dense block removes the launches."""
    nfl = 400
    fptr = list(range(nfl + 1))
    ef, eb = [1] * nfl, [1] * nfl
    plan = _plan(fptr, ef, eb, 4, 32768, 100e-6)
    assert plan and any(d for _, _, d in plan)
