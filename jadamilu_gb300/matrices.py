"""Seeded generators for the test and benchmark matrices.

Every generator returns the matrix in the storage the JADAMILU drivers take
(reference ``src/jd/PJD.F:39-70``): a 1-based CSR of the upper triangle, each
off-diagonal entry stored once, every diagonal entry present and stored first in
its row.  Arrays are ``int32`` (``ia``, ``ja``) and ``float64`` or
``complex128`` (``a``).

The generators follow the reference sample programs where one exists:

* ``tridiag``: the N=1000 matrices of ``samples/EXAMPLE1.f:35-47`` (and the
  EXAMPLE2..11 variants, which only change the diagonal);
* ``laplace3d``: ``MakeLaplaceMatrix`` in ``samples/laplace.f:122-193``;
* ``anderson3d``: ``MakeAndersonMatrix`` in ``samples/anderson.f:113-164``,
  with the reference's libc ``rand()`` replaced by a seeded splitmix64 stream
  and hopping -1 (the spectrum is the same: an even periodic cubic lattice is
  bipartite, so the gauge (-1)^(x+y+z) flips the hopping sign);
* ``tight_binding3d`` and ``fem_p1`` have no reference sample; they build the
  complex Hermitian and generalized workloads with the sizes quoted for them.
"""
from __future__ import annotations

import numpy as np

_MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_uniform(seed: int, count: int) -> np.ndarray:
    """``count`` doubles uniform in [0, 1) from a splitmix64 stream.

    splitmix64 (Steele, Lea, Flood 2014): state += 0x9E3779B97F4A7C15, then
    two xor-shift-multiply rounds; the top 53 bits give the double.
    """
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = (np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)) & _MASK
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _coo_upper_to_csr(n, rows, cols, vals, diag, dtype):
    """Upper CSR, 1-based, diagonal first, from strictly-upper COO + diagonal."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=dtype)
    assert np.all(rows < cols)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    counts = np.bincount(rows, minlength=n) + 1
    ia = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=ia[1:])
    nnz = int(ia[-1])
    ja = np.empty(nnz, dtype=np.int64)
    a = np.empty(nnz, dtype=dtype)
    ja[ia[:-1]] = np.arange(n)
    a[ia[:-1]] = np.asarray(diag, dtype=dtype)
    # off-diagonals follow the diagonal in each row
    start = np.repeat(ia[:-1] + 1, counts - 1)
    within = np.arange(len(rows)) - np.repeat(np.cumsum(counts - 1) - (counts - 1), counts - 1)
    pos = start + within
    ja[pos] = cols
    a[pos] = vals
    return (ia + 1).astype(np.int32), (ja + 1).astype(np.int32), a


def tridiag(n: int = 1000, diag_offset: float = -1.0, diag_scale: float = 1.0,
            off: float = 5.0):
    """a_ii = diag_scale*(i + diag_offset) (1-based i), a_i,i+1 = off.

    EXAMPLE1/2 use diag_offset=-1 (a_ii = i-1); EXAMPLE9/10/11 use
    diag_offset=0 (a_ii = i); EXAMPLE5/6 use diag_scale=0 (a_ii = 0).
    """
    i = np.arange(1, n + 1, dtype=np.float64)
    diag = diag_scale * (i + diag_offset)
    rows = np.arange(n - 1)
    return _coo_upper_to_csr(n, rows, rows + 1, np.full(n - 1, off), diag, np.float64)


def laplace3d(m: int):
    """7-point Dirichlet Laplacian on an m^3 grid scaled by (m+1)^2."""
    n = m ** 3
    h2 = float((m + 1) * (m + 1))
    idx = np.arange(n)
    i, j, k = idx % m, (idx // m) % m, idx // (m * m)
    rows, cols = [], []
    for mask, step in ((i < m - 1, 1), (j < m - 1, m), (k < m - 1, m * m)):
        rows.append(idx[mask])
        cols.append(idx[mask] + step)
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    return _coo_upper_to_csr(n, rows, cols, np.full(len(rows), -h2),
                             np.full(n, 6.0 * h2), np.float64)


def laplace3d_eigenvalues(m: int, count: int) -> np.ndarray:
    """The ``count`` smallest eigenvalues of ``laplace3d(m)`` (closed form)."""
    h2 = float((m + 1) * (m + 1))
    mu = 2.0 * (1.0 - np.cos(np.arange(1, m + 1) * np.pi / (m + 1)))
    s = (mu[:, None, None] + mu[None, :, None] + mu[None, None, :]).ravel()
    return np.sort(s)[:count] * h2


def anderson3d(m: int, disorder: float = 16.5, seed: int = 0, hopping: float = -1.0,
               periodic: bool = True):
    """3-D Anderson model on an m^3 lattice, diagonal U[-W/2, W/2]."""
    n = m ** 3
    idx = np.arange(n, dtype=np.int64)
    i, j, k = idx % m, (idx // m) % m, idx // (m * m)
    diag = (splitmix64_uniform(seed, n) - 0.5) * disorder
    rows, cols = [], []
    for axis, step in ((i, 1), (j, m), (k, m * m)):
        if periodic:
            nb = np.where(axis < m - 1, idx + step, idx - (m - 1) * step)
            sel = np.ones(n, dtype=bool)
        else:
            nb = idx + step
            sel = axis < m - 1
        p, q = idx[sel], nb[sel]
        rows.append(np.minimum(p, q))
        cols.append(np.maximum(p, q))
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    if periodic and m <= 2:
        raise ValueError("periodic lattice needs m >= 3")
    return _coo_upper_to_csr(n, rows, cols, np.full(len(rows), hopping), diag, np.float64)


def tight_binding3d(m: int, phi: float = 1.0 / 17.0, disorder: float = 4.0, seed: int = 1,
                    hopping: float = -1.0):
    """Complex Hermitian tight-binding model, open boundaries.

    Hops along x and z carry ``hopping``; the hop from (x, y, z) to
    (x, y+1, z) carries ``hopping * exp(2 pi i phi x)`` (a Peierls phase of a
    uniform field along z).  On-site energies U[-W/2, W/2].
    """
    n = m ** 3
    idx = np.arange(n, dtype=np.int64)
    i, j, k = idx % m, (idx // m) % m, idx // (m * m)
    diag = (splitmix64_uniform(seed, n) - 0.5) * disorder
    rows, cols, vals = [], [], []
    for axis, step, phased in ((i, 1, False), (j, m, True), (k, m * m, False)):
        sel = axis < m - 1
        p = idx[sel]
        rows.append(p)
        cols.append(p + step)
        if phased:
            # H[q, p] = t e^{i 2 pi phi x}; stored entry is H[p, q] = conj
            vals.append(hopping * np.exp(-2j * np.pi * phi * i[sel]))
        else:
            vals.append(np.full(len(p), hopping, dtype=np.complex128))
    return _coo_upper_to_csr(n, np.concatenate(rows), np.concatenate(cols),
                             np.concatenate(vals), diag.astype(np.complex128), np.complex128)


def fem_p1(m: int, sigma: float = 0.5, seed: int = 3):
    """P1 stiffness K and lumped mass M on an m x m node grid of the unit square.

    Each grid cell is split into two triangles along its diagonal; element e has
    conductivity exp(sigma * g_e) with g_e standard normal (Box-Muller on the
    splitmix64 stream).  Boundary nodes are removed (homogeneous Dirichlet), so
    the unknowns are the (m-2)^2 interior nodes.  Returns (K, M) as upper CSR
    triples; M is diagonal.
    """
    h = 1.0 / (m - 1)
    ncell = (m - 1) * (m - 1)
    u = splitmix64_uniform(seed, 2 * ncell)
    u1 = np.maximum(u[0::2], 1e-300)
    g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u[1::2])
    # two triangles per cell: lower (nodes a,b,c) and upper (a,c,d) share kappa rows
    gx = np.concatenate([g, g[::-1]])  # second triangle takes a different draw order
    kappa = np.exp(sigma * gx)
    cx, cy = np.meshgrid(np.arange(m - 1), np.arange(m - 1), indexing="xy")
    cx, cy = cx.ravel(), cy.ravel()
    n00 = cy * m + cx
    n10 = n00 + 1
    n01 = n00 + m
    n11 = n01 + 1
    tris = np.concatenate([np.stack([n00, n10, n11], 1), np.stack([n00, n11, n01], 1)])
    xy = np.stack([np.tile(np.arange(m), m) * h, np.repeat(np.arange(m), m) * h], 1)
    P = xy[tris]                                   # (ne, 3, 2)
    d1 = P[:, 1] - P[:, 0]
    d2 = P[:, 2] - P[:, 0]
    area = 0.5 * np.abs(d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0])
    # gradients of the barycentric functions
    G = np.empty((len(tris), 3, 2))
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        e = P[:, c] - P[:, b]
        G[:, a, 0] = e[:, 1]
        G[:, a, 1] = -e[:, 0]
    G /= (2.0 * area)[:, None, None]
    sign = np.sign(np.einsum("ni,ni->n", G[:, 0], P[:, 0] - P[:, 1]))
    G *= sign[:, None, None]
    Ke = kappa[:, None, None] * area[:, None, None] * np.einsum("nad,nbd->nab", G, G)
    nn = m * m
    interior = np.zeros(nn, dtype=bool)
    ix, iy = np.arange(nn) % m, np.arange(nn) // m
    interior[(ix > 0) & (ix < m - 1) & (iy > 0) & (iy < m - 1)] = True
    newid = -np.ones(nn, dtype=np.int64)
    newid[interior] = np.arange(interior.sum())
    n = int(interior.sum())
    r = newid[np.repeat(tris, 3, axis=1).ravel()]
    c = newid[np.tile(tris, (1, 3)).ravel()]
    v = Ke.ravel()
    keep = (r >= 0) & (c >= 0) & (r <= c)
    r, c, v = r[keep], c[keep], v[keep]
    key = r * n + c
    uniq, inv = np.unique(key, return_inverse=True)
    vals = np.bincount(inv, weights=v)
    ur, uc = uniq // n, uniq % n
    dmask = ur == uc
    diag = np.zeros(n)
    diag[ur[dmask]] = vals[dmask]
    K = _coo_upper_to_csr(n, ur[~dmask], uc[~dmask], vals[~dmask], diag, np.float64)
    # lumped mass: each element gives area/3 to each of its vertices
    lump = np.bincount(tris.ravel(), weights=np.repeat(area / 3.0, 3), minlength=nn)
    M = _coo_upper_to_csr(n, np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0),
                          lump[interior], np.float64)
    return K, M


def to_scipy_full(ia, ja, a):
    """Full (both triangles) scipy CSR of an upper-stored 1-based matrix."""
    import scipy.sparse as sp
    n = len(ia) - 1
    rows = np.repeat(np.arange(n), np.diff(ia))
    cols = np.asarray(ja, dtype=np.int64) - 1
    U = sp.csr_matrix((a, (rows, cols)), shape=(n, n))
    off = sp.triu(U, k=1)
    return (sp.diags(U.diagonal()) + off + off.conj().T).tocsr()
