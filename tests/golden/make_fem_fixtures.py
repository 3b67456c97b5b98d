"""Golden eigenvalues of the generalized FEM workload.

Matrices: P1 stiffness K and lumped mass M on a structured triangulation of
the unit square with m x m nodes (Dirichlet boundary removed: n = (m - 2)^2),
lognormal conductivity (sigma 0.5) from the seeded splitmix64 stream (seed
3), as the benchmark builds them.  Problem K x = lambda M x, the 6 smallest
eigenvalues (ISEARCH = 0), MADSPACE = 20, TOL 1e-10, DROPTOL 1e-3, MEM 20,
float64 factor: the benchmark's settings.

Recorded at m = 128 and m = 512 (n = 260,100): the CPU oracle's eigenvalues
(the reference's algorithm restated, with the project's factor) and those of
scipy's shift-and-invert Lanczos at sigma = 0 (ARPACK on a sparse LU of K),
which shares no code with this repository.

Run from the repository root (about a minute on one host):

    python tests/golden/make_fem_fixtures.py
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

KW = dict(isearch=0, sigma=0.0, madspace=20, maxit=100000, tol=1e-10, droptol=1e-3, mem=20.0, icntl=(0, 1, 0, 0, 0))


def main():
    import scipy.sparse.linalg as sla
    from jadamilu_gb300 import matrices as M
    import oracle_lib
    out = {"matrix": "fem_p1(m, sigma=0.5, seed=3): K x = lambda M x, lumped M", "neig": 6,
           "settings": {k: (list(v) if isinstance(v, tuple) else v) for k, v in KW.items()}, "cases": {}}
    for m in (128, 512):
        K, Mm = M.fem_p1(m, sigma=0.5, seed=3)
        case = {"n": len(K[0]) - 1}
        t = time.time()
        w = sla.eigsh(M.to_scipy_full(*K).tocsc(), k=6, M=M.to_scipy_full(*Mm).tocsc(), sigma=0.0, which="LM",
                      tol=1e-14, return_eigenvectors=False)
        case["shift_invert"] = np.sort(w).tolist()
        print(f"{m}^2 shift-invert {time.time() - t:.1f} s", flush=True)
        t = time.time()
        r = oracle_lib.dpjd(*K, 6, b=Mm, **KW)
        assert r["info"] == 0 and r["neig"] == 6, (r["info"], r["neig"])
        case["oracle"] = np.sort(r["eigs"]).tolist()
        case["oracle_matvec"] = r["iter"]
        print(f"{m}^2 oracle {time.time() - t:.1f} s, {r['iter']} MATVECs", flush=True)
        out["cases"][str(m)] = case
        with open(os.path.join(HERE, "fem_eigs.json"), "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
