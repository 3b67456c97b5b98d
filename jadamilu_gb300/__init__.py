"""GB300 Jacobi-Davidson eigensolver with the JADAMILU driver interface.

The compute path is the in-tree CUDA library ``_lib/libjadamilu_gb300.so``
(sm_103a kernels behind a C ABI, see ``include/jadamilu_gb300.h``).  This
module only loads it and mirrors the reference drivers for Python callers:

* :func:`dpjd` / :func:`zpjd`      -- DPJD / ZPJD (built-in matvec and
  preconditioner), and the ``_gep`` forms;
* :func:`dpjdrevcom` / :func:`djdrevcom` -- the reverse-communication
  drivers, driven by Python callables for the matvec (and preconditioner);
* :func:`dpjdcleanup` / :func:`zpjdcleanup`.

Arguments mean what they mean in the reference (src/jd/PJD.F): matrices are
upper (or lower) triangles in 1-based CSR with every diagonal entry present;
``icntl`` is ICNTL(1..5); the workspace length follows PJD.F:99-103.  There
is no CPU fallback: without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libjadamilu_gb300.so")

_lib = None
_P = C.c_void_p
_I = C.POINTER(C.c_int)
_D = C.POINTER(C.c_double)


def load(build_if_missing: bool = True):
    """Load (and if needed build) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library missing: {LIB_PATH}")
        from . import build
        build.build_gpu()
    _lib = C.CDLL(LIB_PATH)
    L = _lib
    pjd_args = [_P] * 22
    for name in ("dpjd_", "zpjd_", "pjd_"):
        getattr(L, name).argtypes = pjd_args
    L.pjdrevcom_.argtypes = [_P] * 25
    L.jdrevcom_.argtypes = [_P] * 18
    L.pjdcleanup_.argtypes = []
    for name in ("dpjd_gep_", "zpjd_gep_"):
        getattr(L, name).argtypes = [_P] * 25
    for name in ("dpjdrevcom_", "zpjdrevcom_"):
        getattr(L, name).argtypes = [_P] * 25
    for name in ("dpjdrevcom_gep_", "zpjdrevcom_gep_"):
        getattr(L, name).argtypes = [_P] * 29
    for name in ("djdrevcom_", "zjdrevcom_"):
        getattr(L, name).argtypes = [_P] * 18
    for name in ("djdrevcom_gep_", "zjdrevcom_gep_"):
        getattr(L, name).argtypes = [_P] * 19
    L.dpjdcleanup_.argtypes = []
    L.zpjdcleanup_.argtypes = []
    L.jdgpu_device_count.restype = C.c_int
    L.jdgpu_dspmv.argtypes = [C.c_int, _P, _P, _P, _P, _P]
    L.jdgpu_zspmv.argtypes = [C.c_int, _P, _P, _P, _P, _P]
    L.jdgpu_dildl_apply.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.c_int, _P, _P, _P]
    L.jdgpu_set_option.argtypes = [C.c_char_p, C.c_double]
    L.jdgpu_revcom_device_ptr.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.jdgpu_revcom_device_ptr.restype = C.c_int
    L.jdgpu_deig_grad.argtypes = [C.c_int, _P, _P, C.c_int, _P, C.c_int, _P, _P, _P]
    L.jdgpu_dildl_bench.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.c_int, _P]
    L.jdgpu_dprepare_matrix.argtypes = [C.c_int, _P, _P, _P]
    L.jdgpu_drelease_matrix.argtypes = []
    L.jdgpu_dmatrix_info.argtypes = [_P]
    L.jdgpu_set_stream.argtypes = [_P]
    L.jdgpu_dstats.argtypes = [_P]
    L.jdgpu_zstats.argtypes = [_P]
    L.jdgpu_reset_stats.argtypes = []
    return L


def _require_gpu(L):
    if L.jdgpu_device_count() <= 0:
        raise RuntimeError("jadamilu_gb300: no CUDA device visible; this library has no CPU path")


def _p(a):
    return None if a is None else a.ctypes.data_as(_P)


def lx_required(n: int, neig: int, madspace: int, gep: bool = False) -> int:
    """Workspace length recommended by PJD.F:99-103 (with room for GEP)."""
    return n * (3 * madspace + 2 * neig + 4) + 4 * madspace * madspace + max(madspace * madspace, neig)


class _Args:
    """Fortran-style by-reference argument block."""

    def __init__(self, n, neig, sigma, isearch, ninit, madspace, maxit, tol, shift, droptol, mem, icntl, iprint,
                 dtype, x=None, eigs=None, lx=None):
        self.n = np.array([n], np.int32)
        self.lx_val = lx if lx is not None else lx_required(n, neig, madspace)
        self.lx = np.array([self.lx_val], np.int32)
        self.X = np.zeros(self.lx_val, dtype)
        if x is not None:
            xv = np.asarray(x, dtype)
            flat = xv.T.ravel() if xv.ndim > 1 else xv
            self.X[:flat.size] = flat
        self.EIGS = np.zeros(max(neig, 1), np.float64)
        if eigs is not None:
            self.EIGS[:len(eigs)] = eigs
        self.RES = np.zeros(max(neig, 1), np.float64)
        self.NEIG = np.array([neig], np.int32)
        self.SIGMA = np.array([sigma], np.float64)
        self.ISEARCH = np.array([isearch], np.int32)
        self.NINIT = np.array([ninit], np.int32)
        self.MADSPACE = np.array([madspace], np.int32)
        self.ITER = np.array([maxit], np.int32)
        self.TOL = np.array([tol], np.float64)
        self.SHIFT = np.array([shift], np.float64)
        self.DROPTOL = np.array([droptol], np.float64)
        self.MEM = np.array([mem], np.float64)
        self.ICNTL = np.array(list(icntl) + [0] * (5 - len(icntl)), np.int32)
        self.IPRINT = np.array([iprint], np.int32)
        self.INFO = np.zeros(1, np.int32)
        self.GAP = np.zeros(1, np.float64)
        self.IJOB = np.zeros(1, np.int32)
        self.NDX = np.zeros(3, np.int32)

    def result(self, n):
        k = int(self.NEIG[0])
        kk = k + (1 if self.INFO[0] > 0 else 0)
        kk = max(0, min(kk, len(self.EIGS)))
        return dict(eigs=self.EIGS[:k].copy(), res=self.RES[:k].copy(),
                    x=self.X[:n * kk].reshape(kk, n).T.copy() if kk else np.zeros((n, 0)), neig=k,
                    iter=int(self.ITER[0]), info=int(self.INFO[0]), gap=float(self.GAP[0]),
                    shift=float(self.SHIFT[0]), droptol=float(self.DROPTOL[0]), X=self.X)


def _matrix(A, dtype):
    a, ja, ia = A
    return (np.ascontiguousarray(a, dtype), np.ascontiguousarray(ja, np.int32), np.ascontiguousarray(ia, np.int32))


def _pjd(complex_, A, neig, sigma=0.0, isearch=0, ninit=0, madspace=20, maxit=1000, tol=1e-10, shift=0.0,
         droptol=1e-3, mem=20.0, icntl=(0, 0, 0, 0, 0), iprint=0, x=None, eigs=None, B=None, legacy=False):
    L = load()
    _require_gpu(L)
    dt = np.complex128 if complex_ else np.float64
    a, ja, ia = _matrix(A, dt)
    n = len(ia) - 1
    s = _Args(n, neig, sigma, isearch, ninit, madspace, maxit, tol, shift, droptol, mem, icntl, iprint, dt, x, eigs)
    pre = "z" if complex_ else "d"
    common = [_p(s.EIGS), _p(s.RES), _p(s.X), _p(s.lx), _p(s.NEIG), _p(s.SIGMA), _p(s.ISEARCH), _p(s.NINIT),
              _p(s.MADSPACE), _p(s.ITER), _p(s.TOL), _p(s.SHIFT), _p(s.DROPTOL), _p(s.MEM), _p(s.ICNTL)]
    if B is None:
        name = "pjd_" if legacy else pre + "pjd_"
        getattr(L, name)(_p(s.n), _p(a), _p(ja), _p(ia), *common, _p(s.IPRINT), _p(s.INFO), _p(s.GAP))
    else:
        b, jb, ib = _matrix(B, dt)
        getattr(L, pre + "pjd_gep_")(_p(s.n), _p(a), _p(ja), _p(ia), _p(b), _p(jb), _p(ib), *common, _p(s.IPRINT),
                                     _p(s.INFO), _p(s.GAP))
    out = s.result(n)
    out.update(a=a, ja=ja, ia=ia, icntl=s.ICNTL.copy())
    return out


def dpjd(A, neig, **kw):
    """DPJD: eigenpairs of the real symmetric matrix A = (a, ja, ia)."""
    return _pjd(False, A, neig, **kw)


def zpjd(A, neig, **kw):
    """ZPJD: eigenpairs of the complex Hermitian matrix A = (a, ja, ia)."""
    return _pjd(True, A, neig, **kw)


def dpjd_gep(A, B, neig, **kw):
    """DPJD_GEP: A x = lambda B x with B symmetric positive definite."""
    return _pjd(False, A, neig, B=B, **kw)


def zpjd_gep(A, B, neig, **kw):
    """ZPJD_GEP: A x = lambda B x with complex Hermitian A and Hermitian positive definite B."""
    return _pjd(True, A, neig, B=B, **kw)


def _revcom(complex_, kind, A, neig, matvec, precond=None, sigma=0.0, isearch=0, ninit=0, madspace=20, maxit=1000,
            tol=1e-10, shift=0.0, droptol=1e-3, mem=20.0, icntl=(0, 0, 0, 0, 0), iprint=0, x=None, eigs=None, n=None,
            B=None, bmatvec=None, device=False):
    """Reverse-communication loop: serves IJOB requests with Python callables.

    Host mode: ``matvec(x) -> A x``, ``bmatvec(x) -> B x``, ``precond(r) -> z``
    on numpy vectors.  Device mode (``device=True``, jdgpu_revcom_device_ptr):
    the callables get device addresses and serve the request on the GPU,
    ``matvec(x_addr, y_addr, n, stream)``, ``bmatvec(x_addr, y_addr, n, stream)``,
    ``precond(r_addr, z_addr, n, stream)``; their results must be complete (or
    enqueued on ``stream``) when they return."""
    L = load()
    _require_gpu(L)
    item = 16 if complex_ else 8
    first = True
    dt = np.complex128 if complex_ else np.float64
    pre = "z" if complex_ else "d"
    if A is not None:
        a, ja, ia = _matrix(A, dt)
        n = len(ia) - 1
    s = _Args(n, neig, sigma, isearch, ninit, madspace, maxit, tol, shift, droptol, mem, icntl, iprint, dt, x, eigs)
    X = s.X
    gep = B is not None or bmatvec is not None
    if kind == "pjd" and gep:
        b, jb, ib = _matrix(B, dt)
    while True:
        if first and device:  # the mode is taken when the solve starts (IJOB = 0)
            L.jdgpu_set_option(b"revcom_device", C.c_double(1.0))
        if kind == "pjd":
            if gep:
                getattr(L, pre + "pjdrevcom_gep_")(
                    _p(s.n), _p(a), _p(ja), _p(ia), _p(b), _p(jb), _p(ib), _p(s.EIGS), _p(s.RES), _p(X), _p(s.lx),
                    _p(s.NEIG), _p(s.SIGMA), _p(s.ISEARCH), _p(s.NINIT), _p(s.MADSPACE), _p(s.ITER), _p(s.TOL),
                    _p(s.SHIFT), _p(s.DROPTOL), _p(s.MEM), _p(s.ICNTL), _p(s.IJOB), _p(s.NDX[0:1]), _p(s.NDX[1:2]),
                    _p(s.NDX[2:3]), _p(s.IPRINT), _p(s.INFO), _p(s.GAP))
            else:
                getattr(L, pre + "pjdrevcom_")(
                    _p(s.n), _p(a), _p(ja), _p(ia), _p(s.EIGS), _p(s.RES), _p(X), _p(s.lx), _p(s.NEIG), _p(s.SIGMA),
                    _p(s.ISEARCH), _p(s.NINIT), _p(s.MADSPACE), _p(s.ITER), _p(s.TOL), _p(s.SHIFT), _p(s.DROPTOL),
                    _p(s.MEM), _p(s.ICNTL), _p(s.IJOB), _p(s.NDX[0:1]), _p(s.NDX[1:2]), _p(s.IPRINT), _p(s.INFO),
                    _p(s.GAP))
        else:
            if gep:
                getattr(L, pre + "jdrevcom_gep_")(
                    _p(s.n), _p(s.EIGS), _p(s.RES), _p(X), _p(s.lx), _p(s.NEIG), _p(s.SIGMA), _p(s.ISEARCH),
                    _p(s.NINIT), _p(s.MADSPACE), _p(s.ITER), _p(s.TOL), _p(s.IJOB), _p(s.NDX[0:1]), _p(s.NDX[1:2]),
                    _p(s.NDX[2:3]), _p(s.IPRINT), _p(s.INFO), _p(s.GAP))
            else:
                getattr(L, pre + "jdrevcom_")(
                    _p(s.n), _p(s.EIGS), _p(s.RES), _p(X), _p(s.lx), _p(s.NEIG), _p(s.SIGMA), _p(s.ISEARCH),
                    _p(s.NINIT), _p(s.MADSPACE), _p(s.ITER), _p(s.TOL), _p(s.IJOB), _p(s.NDX[0:1]), _p(s.NDX[1:2]),
                    _p(s.IPRINT), _p(s.INFO), _p(s.GAP))
        if first and device:
            L.jdgpu_set_option(b"revcom_device", C.c_double(0.0))
        first = False
        ijob = int(s.IJOB[0])
        if ijob == 0:
            break
        i1, i2, i3 = (int(v) - 1 for v in s.NDX)
        if device:
            xd, st = C.c_void_p(), C.c_void_p()
            if L.jdgpu_revcom_device_ptr(int(complex_), C.byref(xd), C.byref(st)) != 0:
                raise RuntimeError("no device-mode request pending")
            base, stream = int(xd.value), int(st.value or 0)
            if ijob in (1, 3):
                matvec(base + i1 * item, base + i2 * item, n, stream)
            if gep and ijob in (1, 4):
                bmatvec(base + i1 * item, base + i3 * item, n, stream)
            if ijob == 2:
                precond(base + i2 * item, base + i1 * item, n, stream)
            continue
        if ijob in (1, 3):
            X[i2:i2 + n] = matvec(X[i1:i1 + n].copy())
        if gep and ijob in (1, 4):
            X[i3:i3 + n] = bmatvec(X[i1:i1 + n].copy())
        if ijob == 2:
            X[i1:i1 + n] = precond(X[i2:i2 + n].copy())
    return s.result(n)


def dpjdrevcom(A, neig, matvec, **kw):
    """DPJDREVCOM with the matvec served by ``matvec(x) -> A x``."""
    return _revcom(False, "pjd", A, neig, matvec, **kw)


def zpjdrevcom(A, neig, matvec, **kw):
    return _revcom(True, "pjd", A, neig, matvec, **kw)


def djdrevcom(n, neig, matvec, precond, **kw):
    """DJDREVCOM with user matvec and user preconditioner."""
    return _revcom(False, "jd", None, neig, matvec, precond, n=n, **kw)


def zjdrevcom(n, neig, matvec, precond, **kw):
    return _revcom(True, "jd", None, neig, matvec, precond, n=n, **kw)


def dpjdcleanup():
    load().dpjdcleanup_()


def zpjdcleanup():
    load().zpjdcleanup_()


def spmv(A, x):
    """One GPU SpMV y = A x (the built-in matvec kernel)."""
    L = load()
    _require_gpu(L)
    cplx = np.iscomplexobj(A[0]) or np.iscomplexobj(x)
    dt = np.complex128 if cplx else np.float64
    a, ja, ia = _matrix(A, dt)
    x = np.ascontiguousarray(x, dt)
    y = np.zeros_like(x)
    r = (L.jdgpu_zspmv if cplx else L.jdgpu_dspmv)(len(ia) - 1, _p(ia), _p(ja), _p(a), _p(x), _p(y))
    if r != 0:
        raise RuntimeError("GPU SpMV failed")
    return y


def ildl_apply(A, b, shift=0.0, droptol=1e-3, condest=5.0, spd=False, precision=0):
    """Host ILDLC factor of A - shift*I applied on the GPU to the columns of b."""
    L = load()
    _require_gpu(L)
    a, ja, ia = _matrix(A, np.float64)
    n = len(ia) - 1
    b = np.asarray(b, np.float64)
    B = np.ascontiguousarray(b.reshape(-1, n))
    X = np.zeros_like(B)
    info = np.zeros(5, np.int64)
    r = L.jdgpu_dildl_apply(n, _p(ia), _p(ja), _p(a), shift, droptol, condest, int(spd), int(precision), B.shape[0],
                            _p(B), _p(X), _p(info))
    if r != 0:
        raise RuntimeError(f"GPU ILDL apply failed ({r})")
    keys = ["nnz_l", "nneg", "nlevels", "fwd_depth", "bwd_depth"]
    return X.reshape(b.shape), dict(zip(keys, info.tolist()))


def dpjd_batch(problems, neig, workers=8, sigma=0.0, isearch=2, madspace=20, maxit=10000, tol=1e-10,
               droptol=1e-3, mem=20.0, icntl=(0, 0, 0, 0, 1)):
    """Solve independent real symmetric problems [(a, ja, ia), ...] with
    jdgpu_dpjd_batch (worker threads with their own solver state and CUDA
    stream).  Returns one result dict per problem (eigs, res, x, neig, iter,
    info, gap)."""
    L = load()
    _require_gpu(L)
    P = len(problems)
    mats = [_matrix(A, np.float64) for A in problems]
    n = np.array([len(m[2]) - 1 for m in mats], np.int32)
    lx = np.array([k * (3 * madspace + neig + 4) + 3 * madspace * madspace + max(madspace * madspace, neig)
                   for k in n], np.int32)
    X = [np.zeros(int(v)) for v in lx]
    E = [np.zeros(neig) for _ in range(P)]
    R = [np.zeros(neig) for _ in range(P)]
    ptrs = lambda arrs: (C.c_void_p * P)(*[a.ctypes.data for a in arrs])
    NEIG = np.full(P, neig, np.int32)
    ITER = np.full(P, maxit, np.int32)
    INFO = np.zeros(P, np.int32)
    GAP = np.zeros(P)
    ic = np.array(icntl, np.int32)
    L.jdgpu_dpjd_batch.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_double, C.c_int,
                                   C.c_int, C.c_double, C.c_double, C.c_double, _P, C.c_int]
    rc = L.jdgpu_dpjd_batch(P, _p(n), ptrs([m[0] for m in mats]), ptrs([m[1] for m in mats]),
                            ptrs([m[2] for m in mats]), ptrs(E), ptrs(R), ptrs(X), _p(lx), _p(NEIG), _p(ITER),
                            _p(INFO), _p(GAP), sigma, isearch, madspace, tol, droptol, mem, _p(ic), workers)
    if rc != 0:
        raise RuntimeError(f"jdgpu_dpjd_batch failed ({rc})")
    out = []
    for q in range(P):
        k = int(NEIG[q])
        out.append(dict(eigs=E[q][:k].copy(), res=R[q][:k].copy(), x=X[q][:n[q] * k].reshape(k, n[q]).T.copy(),
                        neig=k, iter=int(ITER[q]), info=int(INFO[q]), gap=float(GAP[q])))
    return out


def eig_grad(A, X, w=None, bdiag=None):
    """Gradient of sum_k w[k] * lambda_k with respect to the stored entries of
    A = (a, ja, ia), from eigenvectors X (n x k, columns; any scaling) of
    A x = lambda B x with B = diag(bdiag) or I (jdgpu_deig_grad)."""
    L = load()
    _require_gpu(L)
    a, ja, ia = _matrix(A, np.float64)
    n = len(ia) - 1
    X = np.asfortranarray(np.asarray(X, np.float64).reshape(n, -1))
    k = X.shape[1]
    w = np.ones(k) if w is None else np.ascontiguousarray(w, np.float64)
    bd = None if bdiag is None else np.ascontiguousarray(bdiag, np.float64)
    g = np.zeros(len(a))
    r = L.jdgpu_deig_grad(n, _p(ia), _p(ja), k, _p(X), n, _p(w), _p(bd) if bd is not None else None, _p(g))
    if r != 0:
        raise RuntimeError(f"jdgpu_deig_grad failed ({r})")
    return g


def eigvec_grad(A, lam, x, g, bdiag=None, droptol=1e-3, tol=1e-12, maxit=2000):
    """Gradient of a loss of one eigenvector x (A x = lam B x) with respect to
    the stored entries of A = (a, ja, ia); g = dL/dx at x scaled to
    x^T B x = 1 (jdgpu_deigvec_grad).  Returns (grad, iterations, residual)."""
    L = load()
    _require_gpu(L)
    a, ja, ia = _matrix(A, np.float64)
    n = len(ia) - 1
    x = np.ascontiguousarray(x, np.float64)
    g = np.ascontiguousarray(g, np.float64)
    bd = None if bdiag is None else np.ascontiguousarray(bdiag, np.float64)
    grad = np.zeros(len(a))
    out = np.zeros(2)
    L.jdgpu_deigvec_grad.argtypes = [C.c_int, _P, _P, _P, _P, C.c_double, _P, _P, C.c_double, C.c_double, C.c_int,
                                     _P, _P]
    r = L.jdgpu_deigvec_grad(n, _p(ia), _p(ja), _p(a), _p(bd) if bd is not None else None, lam, _p(x), _p(g),
                             droptol, tol, maxit, _p(grad), _p(out))
    if r != 0:
        raise RuntimeError(f"jdgpu_deigvec_grad failed ({r})")
    return grad, int(out[0]), float(out[1])


def set_option(name: str, value: float) -> None:
    load().jdgpu_set_option(name.encode(), float(value))


def stats(complex_: bool = False) -> dict:
    """Statistics of the last real (or complex) solve."""
    out = np.zeros(12, np.float64)
    L = load()
    (L.jdgpu_zstats if complex_ else L.jdgpu_dstats)(_p(out))
    keys = ["factor_s", "upload_s", "n_precond", "n_matvec", "levels", "fwd_depth", "bwd_depth", "nnz_l", "fill",
            "nfactor", "dense_rows", "dense_blocks"]
    return dict(zip(keys, out.tolist()))


def reset_stats() -> None:
    load().jdgpu_reset_stats()


def ildl_bench(A, shift=0.0, droptol=1e-3, condest=5.0, spd=False, precision=0, reps=20):
    """Time GPU applications of the preconditioner (CUDA events)."""
    L = load()
    _require_gpu(L)
    a, ja, ia = _matrix(A, np.float64)
    out = np.zeros(8, np.float64)
    r = L.jdgpu_dildl_bench(len(ia) - 1, _p(ia), _p(ja), _p(a), shift, droptol, condest, int(spd), int(precision),
                            reps, _p(out))
    if r != 0:
        raise RuntimeError(f"ildl bench failed ({r})")
    keys = ["ms", "nnz_l", "fwd_depth", "bwd_depth", "launches", "factor_s", "tail_rows", "upload_s"]
    return dict(zip(keys, out.tolist()))


def prepare_matrix(A):
    """Upload A once for device-resident solves (see jdgpu_dprepare_matrix)."""
    L = load()
    _require_gpu(L)
    a, ja, ia = _matrix(A, np.float64)
    if L.jdgpu_dprepare_matrix(len(ia) - 1, _p(ia), _p(ja), _p(a)) != 0:
        raise RuntimeError("prepare_matrix failed")


def release_matrix():
    load().jdgpu_drelease_matrix()


def set_stream(handle: int) -> None:
    load().jdgpu_set_stream(C.c_void_p(handle) if handle else None)
