"""ctypes bindings of the CPU oracle (test infrastructure; see oracle/)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

_lib = None

DMV = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double))
DPC = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        _lib = C.CDLL(LIB_PATH)
        p = C.c_void_p
        _lib.orc_dfactor.restype = p
        _lib.orc_dfactor.argtypes = [C.c_int, p, p, p, C.c_double, C.c_double, C.c_double, C.c_double, p]
        _lib.orc_dfactor_info.argtypes = [p, p]
        _lib.orc_dfactor_apply.argtypes = [p, C.c_int, C.c_int, p, p]
        _lib.orc_dfactor_free.argtypes = [p]
        for name in ("orc_dpjd", "orc_zpjd"):
            f = getattr(_lib, name)
            f.argtypes = [C.c_int, p, p, p, p, p, p, p, p, p, C.c_long, p, C.c_double, C.c_int, C.c_int, C.c_int,
                          p, C.c_double, p, p, p, p, p, p, C.c_int, p, p]
        for name in ("orc_djd", "orc_zjd"):
            f = getattr(_lib, name)
            f.argtypes = [C.c_int, p, p, p, C.c_long, p, C.c_double, C.c_int, C.c_int, C.c_int, p, C.c_double,
                          p, p, C.c_int, p, p, p]
        _lib.orc_dmatveca.argtypes = [C.c_int, p, p, p, p, p]
        _lib.orc_zmatveca.argtypes = [C.c_int, p, p, p, p, p]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Factor:
    """Host ILDLC factor (project code) with the oracle's application of it."""

    def __init__(self, ia, ja, a, shift=0.0, droptol=1e-3, condest=5.0, mem=0.0):
        L = lib()
        self.ia, self.ja, self.a = (np.ascontiguousarray(ia, np.int32), np.ascontiguousarray(ja, np.int32),
                                    np.ascontiguousarray(a, np.float64))
        ierr = np.zeros(1, np.int32)
        self.n = len(ia) - 1
        self.h = L.orc_dfactor(self.n, _ptr(self.ia), _ptr(self.ja), _ptr(self.a), shift, droptol, condest, mem,
                               _ptr(ierr))
        self.ierr = int(ierr[0])

    def _check(self):
        if self.ierr != 0:
            raise RuntimeError(f"factorisation failed: ierr={self.ierr}")

    def info(self):
        self._check()
        out = np.zeros(8, np.int64)
        lib().orc_dfactor_info(self.h, _ptr(out))
        keys = ["n", "nnz_l", "nneg", "nlevels", "fwd_depth", "bwd_depth", "n2x2"]
        return dict(zip(keys, out[:7].tolist()))

    def apply(self, b, spd=False, single=False):
        self._check()
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        lib().orc_dfactor_apply(self.h, int(spd), int(single), _ptr(b), _ptr(x))
        return x

    def __del__(self):
        try:
            lib().orc_dfactor_free(self.h)
        except Exception:
            pass


def dpjd(ia, ja, a, neig, sigma=0.0, isearch=0, ninit=0, madspace=20, maxit=1000, tol=1e-10, shift=0.0,
         droptol=1e-3, mem=20.0, icntl=(0, 0, 0, 0, 0), x=None, eigs=None, user_matvec=None, b=None,
         complex_=False):
    """Run the oracle's PJDRVCOM (DPJD, or DPJDREVCOM when user_matvec is given)."""
    L = lib()
    dt = np.complex128 if complex_ else np.float64
    n = len(ia) - 1
    ia = np.array(ia, np.int32)
    ja = np.array(ja, np.int32)
    a = np.array(a, dt)
    gep = b is not None
    lx = n * (3 * madspace + 2 * neig + 4) + 4 * madspace * madspace + max(madspace * madspace, neig)
    X = np.zeros(lx, dt)
    if x is not None:
        X[:x.size] = x.ravel(order="F") if x.ndim > 1 else x
    EIGS = np.zeros(max(neig, 1), np.float64)
    if eigs is not None:
        EIGS[:len(eigs)] = eigs
    RES = np.zeros(max(neig, 1), np.float64)
    NEIG = np.array([neig], np.int32)
    ITER = np.array([maxit], np.int32)
    SHIFT = np.array([shift], np.float64)
    DROPTOL = np.array([droptol], np.float64)
    MEM = np.array([mem], np.float64)
    ICNTL = np.array(icntl, np.int32)
    INFO = np.zeros(1, np.int32)
    GAP = np.zeros(1, np.float64)
    if gep:
        ib, jb, bv = (np.array(b[0], np.int32), np.array(b[1], np.int32), np.array(b[2], dt))
    else:
        ib = jb = bv = None
    cb = None
    if user_matvec is not None:
        def _mv(ctx, which, xp, yp, byp):
            xv = np.ctypeslib.as_array(xp, (n,))
            yv = np.ctypeslib.as_array(yp, (n,))
            yv[:] = user_matvec(xv.copy())
        cb = DMV(_mv)
    f = L.orc_zpjd if complex_ else L.orc_dpjd
    f(n, _ptr(a), _ptr(ja), _ptr(ia), _ptr(bv), _ptr(jb), _ptr(ib), _ptr(EIGS), _ptr(RES), _ptr(X), lx,
      _ptr(NEIG), sigma, isearch, ninit, madspace, _ptr(ITER), tol, _ptr(SHIFT), _ptr(DROPTOL), _ptr(MEM),
      _ptr(ICNTL), _ptr(INFO), _ptr(GAP), int(gep), C.cast(cb, C.c_void_p) if cb else None, None)
    k = int(NEIG[0])
    return dict(eigs=EIGS[:k].copy(), res=RES[:k].copy(), x=X[:n * k].reshape(k, n).T.copy(), neig=k,
                iter=int(ITER[0]), info=int(INFO[0]), gap=float(GAP[0]), shift=float(SHIFT[0]),
                droptol=float(DROPTOL[0]), a=a, ja=ja, ia=ia)
