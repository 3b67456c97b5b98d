"""Golden eigenvalues of the complex Hermitian tight-binding workload.

Matrix: 3-D tight-binding model on an m^3 lattice with open boundaries,
hopping -1, Peierls phases exp(i 2 pi phi x) on the y-hops with phi = 1/17,
on-site energies uniform in [-2, 2] from the seeded splitmix64 stream (seed
1), as the benchmark builds it.  Settings as the benchmark: the 8 smallest
eigenvalues (ISEARCH = 0), MADSPACE = 20, TOL 1e-10, DROPTOL 1e-3, MEM 20,
complex64 factor.

Recorded: the CPU oracle's eigenvalues (the reference's algorithm restated,
with the project's factor) at 32^3 and 64^3, and at 32^3 also those of
scipy's Lanczos (ARPACK, smallest algebraic), which shares no code with this
repository.

Run from the repository root (minutes on one host):

    python tests/golden/make_tightbinding_fixtures.py
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

KW = dict(isearch=0, sigma=0.0, madspace=20, maxit=100000, tol=1e-10, droptol=1e-3, mem=20.0, icntl=(0, 1, 0, 0, 1))


def main():
    import scipy.sparse.linalg as sla
    from jadamilu_gb300 import matrices as M
    import oracle_lib
    out = {"matrix": "tight_binding3d(m, phi=1/17, disorder=4.0, seed=1), open boundaries, hopping -1", "neig": 8,
           "settings": {k: (list(v) if isinstance(v, tuple) else v) for k, v in KW.items()}, "cases": {}}
    for m in (32, 64):
        ia, ja, a = M.tight_binding3d(m, phi=1.0 / 17.0, disorder=4.0, seed=1)
        case = {"n": m ** 3}
        if m <= 32:
            t = time.time()
            w = sla.eigsh(M.to_scipy_full(ia, ja, a).tocsc(), k=8, which="SA", tol=1e-13, return_eigenvectors=False)
            case["lanczos"] = np.sort(w).tolist()
            print(f"{m}^3 Lanczos {time.time() - t:.1f} s", flush=True)
        t = time.time()
        r = oracle_lib.dpjd(ia, ja, a, 8, complex_=True, **KW)
        assert r["info"] == 0 and r["neig"] == 8, (r["info"], r["neig"])
        case["oracle"] = np.sort(r["eigs"]).tolist()
        case["oracle_matvec"] = r["iter"]
        print(f"{m}^3 oracle {time.time() - t:.1f} s, {r['iter']} MATVECs", flush=True)
        out["cases"][str(m)] = case
        with open(os.path.join(HERE, "tightbinding_eigs.json"), "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
