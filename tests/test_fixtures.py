"""The committed golden eigenvalue fixtures (tests/golden/*_eigs.json): the
oracle's values agree with the independent solver recorded beside them
(ARPACK Lanczos or shift-and-invert, no code shared with this repository),
and the oracle reproduces its own recorded values on a case that runs in
under a second."""
import json
import os

import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("name,indep", [("anderson_eigs.json", ("shift_invert", "shift_invert14", "lanczos")),
                                        ("tightbinding_eigs.json", ("lanczos",)),
                                        ("fem_eigs.json", ("shift_invert",))])
def test_oracle_agrees_with_independent_solver(name, indep):
    fx = _load(name)
    checked = 0
    for m, case in fx["cases"].items():
        for key in indep:
            if key not in case or "oracle" not in case:
                continue
            ref = np.sort(np.array(case[key]))
            for lam in case["oracle"]:
                # every oracle eigenvalue is one of the independent solver's
                assert np.min(np.abs(ref - lam)) <= max(1e-10 * abs(lam), 1e-12), (name, m, key, lam)
            checked += 1
    assert checked > 0


def test_oracle_reproduces_fem_fixture(oracle):
    fx = _load("fem_eigs.json")
    st = fx["settings"]
    K, Mm = M.fem_p1(128, sigma=0.5, seed=3)
    r = oracle.dpjd(*K, 6, b=Mm, isearch=st["isearch"], sigma=st["sigma"], madspace=st["madspace"],
                    maxit=st["maxit"], tol=st["tol"], droptol=st["droptol"], mem=st["mem"],
                    icntl=tuple(st["icntl"]))
    assert r["info"] == 0 and r["neig"] == 6
    np.testing.assert_allclose(np.sort(r["eigs"]), fx["cases"]["128"]["oracle"], rtol=1e-10, atol=0)
