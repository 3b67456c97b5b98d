"""Golden eigenvalues of the benchmark's Anderson matrices.

The reference publishes no results for these matrices, so the fixtures come
from two sources:

* shift-and-invert Lanczos (scipy's ARPACK on SuperLU's sparse LU of A),
  which shares no code with this repository, for the 10 eigenvalues closest
  to 0 where the LU fits in memory (40^3);
* the CPU oracle of this repository (the reference's algorithm restated, with
  the project's factor) for the same 10 eigenvalues, with the MATVEC count of
  its complete solve (the reference arm of bench.py scales capped samples to
  it), at every listed size.

Both are also recorded for the 14 eigenvalues closest to 0 (Lanczos at 40^3,
the oracle with NEIG = 14 up to 60^3): a Jacobi-Davidson run can skip one
member of a tight cluster and return the next eigenvalue instead, so the
parity tests check every returned eigenvalue against this wider set.

Matrices: 3-D Anderson model, periodic m^3 lattice, hopping -1, diagonal
uniform in [-8.25, 8.25] from the seeded splitmix64 stream (seed 0), as the
benchmark builds them.  Solver settings as the benchmark: ISEARCH = 2,
sigma = 0, MADSPACE = 25, TOL 1e-10, DROPTOL 1e-3 (the reference's Anderson
sample), MEM 20, float32 factor.

Run from the repository root (sizes as arguments; 100 takes tens of minutes
on one core):

    python tests/golden/make_anderson_fixtures.py 40 60 100
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

KW = dict(isearch=2, sigma=0.0, madspace=25, maxit=100000, tol=1e-10, droptol=1e-3, mem=20.0, icntl=(0, 1, 0, 0, 1))
LANCZOS_MAX = 40  # largest lattice edge whose sparse LU this script factors
ORACLE14_MAX = 60  # largest lattice edge with the 14-eigenvalue oracle solve


def main(sizes):
    from jadamilu_gb300 import matrices as M
    from problems import shift_invert_eigs
    import oracle_lib
    dst = os.path.join(HERE, "anderson_eigs.json")
    out = {"matrix": "anderson3d(m, disorder=16.5, seed=0), periodic, hopping -1", "neig": 10, "sigma": 0.0,
           "settings": {k: (list(v) if isinstance(v, tuple) else v) for k, v in KW.items()}, "cases": {}}
    if os.path.exists(dst):
        with open(dst) as f:
            old = json.load(f)
        if old.get("settings") == out["settings"]:
            out["cases"] = old.get("cases", {})
    for m in sizes:
        ia, ja, a = M.anderson3d(m, disorder=16.5, seed=0)
        case = out["cases"].get(str(m), {"n": m ** 3})
        if m <= LANCZOS_MAX and "shift_invert14" not in case:
            t = time.time()
            w = shift_invert_eigs(M.to_scipy_full(ia, ja, a), 14)
            w = w[np.argsort(np.abs(w), kind="stable")]
            case["shift_invert14"] = np.sort(w).tolist()
            case["shift_invert"] = np.sort(w[:10]).tolist()
            print(f"{m}^3 shift-invert Lanczos {time.time() - t:.1f} s", flush=True)
        if "oracle" not in case:
            t = time.time()
            r = oracle_lib.dpjd(ia, ja, a, 10, **KW)
            assert r["info"] == 0 and r["neig"] == 10, (r["info"], r["neig"])
            case["oracle"] = np.sort(r["eigs"]).tolist()
            case["oracle_matvec"] = r["iter"]
            case["oracle_max_res"] = float(np.max(r["res"]))
            print(f"{m}^3 oracle {time.time() - t:.1f} s, {r['iter']} MATVECs", flush=True)
        if m <= ORACLE14_MAX and "oracle14" not in case:
            t = time.time()
            r = oracle_lib.dpjd(ia, ja, a, 14, **KW)
            assert r["info"] == 0 and r["neig"] == 14, (r["info"], r["neig"])
            case["oracle14"] = np.sort(r["eigs"]).tolist()
            print(f"{m}^3 oracle (14) {time.time() - t:.1f} s, {r['iter']} MATVECs", flush=True)
        out["cases"][str(m)] = case
        with open(dst, "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main([int(v) for v in sys.argv[1:]] or [40, 60])
