"""Device-pointer reverse communication (jdgpu_revcom_device_ptr): the
requests of DPJDREVCOM / DJDREVCOM and their _GEP and Z forms are served by
GPU-resident operators on the library's device copy of X, with no host copy
of the request vectors.  The user operators here are PyTorch CUDA kernels
(CSR matvec, diagonal scaling); the library's vectors reach them through
device-to-device copies."""
import ctypes as C
import os

import numpy as np
import pytest

from jadamilu_gb300 import matrices as M

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

D2D = 3  # cudaMemcpyDeviceToDevice


def _cudart():
    import glob
    cands = [os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart.so*")]
    cands += ["/usr/local/cuda/lib64/libcudart.so*"]
    for pat in cands:
        for path in sorted(glob.glob(pat)):
            try:
                lib = C.CDLL(path)
                lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
                lib.cudaMemcpy.restype = C.c_int
                return lib
            except OSError:
                continue
    pytest.skip("libcudart not found")


class DeviceOps:
    """A, B (diagonal) and a diagonal preconditioner as CUDA tensors; each
    request copies the library's input vector into a tensor, computes, and
    copies the result back, all on the device."""

    def __init__(self, ia, ja, a, dtype, bdiag=None, pdiag=None):
        self.rt = _cudart()
        As = M.to_scipy_full(ia, ja, a).tocsr()
        dev = torch.device("cuda")
        self.A = torch.sparse_csr_tensor(torch.tensor(As.indptr, dtype=torch.int64), torch.tensor(As.indices,
                                         dtype=torch.int64), torch.tensor(As.data, dtype=dtype), size=As.shape,
                                         device=dev)
        self.b = None if bdiag is None else torch.tensor(bdiag, dtype=dtype, device=dev)
        self.p = None if pdiag is None else torch.tensor(pdiag, dtype=dtype, device=dev)
        self.dtype, self.dev = dtype, dev
        self.calls = 0

    def _get(self, addr, n):
        t = torch.empty(n, dtype=self.dtype, device=self.dev)
        torch.cuda.synchronize()
        assert self.rt.cudaMemcpy(t.data_ptr(), addr, t.element_size() * n, D2D) == 0
        return t

    def _put(self, addr, t):
        torch.cuda.synchronize()
        assert self.rt.cudaMemcpy(addr, t.data_ptr(), t.element_size() * t.numel(), D2D) == 0

    def matvec(self, x, y, n, stream):
        self.calls += 1
        self._put(y, torch.matmul(self.A, self._get(x, n)))

    def bmatvec(self, x, y, n, stream):
        self._put(y, self.b * self._get(x, n))

    def precond(self, r, z, n, stream):
        self._put(z, self._get(r, n) / self.p)


def test_dpjdrevcom_device_anderson(gpu):
    ia, ja, a = M.anderson3d(10, seed=5)
    ops = DeviceOps(ia, ja, a, torch.float64)
    kw = dict(sigma=0.0, isearch=2, madspace=20, maxit=5000, tol=1e-10, droptol=1e-3)
    r = gpu.dpjdrevcom((a.copy(), ja.copy(), ia.copy()), 4, ops.matvec, device=True, **kw)
    assert r["info"] == 0 and r["neig"] == 4 and ops.calls == r["iter"]
    w = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a).toarray())
    ref = np.sort(w[np.argsort(np.abs(w))[:4]])
    np.testing.assert_allclose(np.sort(r["eigs"]), ref, rtol=1e-9, atol=1e-12)
    # eigenvectors come back in the caller's X as in host mode
    As = M.to_scipy_full(ia, ja, a)
    for k in range(4):
        v = r["x"][:, k]
        assert np.linalg.norm(As @ v - r["eigs"][k] * v) <= 1e-9 * np.linalg.norm(v)


def test_djdrevcom_device_with_device_preconditioner(gpu):
    """DJDREVCOM with a user matvec and a user (diagonal) preconditioner, both
    on the device: valid eigenpairs, and the eigenvalues of host-mode
    DJDREVCOM with the same operators."""
    ia, ja, a = M.anderson3d(8, seed=7)
    n = 8 ** 3
    As = M.to_scipy_full(ia, ja, a)
    p = np.abs(As.diagonal()) + 1.0
    ops = DeviceOps(ia, ja, a, torch.float64, pdiag=p)
    kw = dict(isearch=0, madspace=20, maxit=20000, tol=1e-10)
    r = gpu.djdrevcom(n, 5, ops.matvec, ops.precond, device=True, **kw)
    assert r["info"] == 0 and r["neig"] == 5
    host = gpu.djdrevcom(n, 5, lambda x: As @ x, lambda v: v / p, **kw)
    assert host["info"] == 0
    np.testing.assert_allclose(np.sort(r["eigs"]), np.sort(host["eigs"]), rtol=1e-9, atol=1e-12)
    w = np.linalg.eigvalsh(As.toarray())
    for lam in r["eigs"]:
        assert np.min(np.abs(w - lam)) <= 1e-9 * max(1.0, abs(lam))
    for k in range(5):
        v = r["x"][:, k]
        assert np.linalg.norm(As @ v - r["eigs"][k] * v) <= 1e-9 * np.linalg.norm(v)


def test_dpjdrevcom_gep_device_fem(gpu):
    K, Mm = M.fem_p1(12, seed=3)
    md = M.to_scipy_full(*Mm).toarray().diagonal()
    ops = DeviceOps(*K, torch.float64, bdiag=md)
    r = gpu.dpjdrevcom((K[2].copy(), K[1].copy(), K[0].copy()), 4, ops.matvec, B=(Mm[2], Mm[1], Mm[0]),
                       bmatvec=ops.bmatvec, isearch=0, madspace=20, maxit=4000, tol=1e-10, droptol=1e-3,
                       device=True)
    assert r["info"] == 0 and r["neig"] == 4
    import scipy.linalg as sl
    w = sl.eigh(M.to_scipy_full(*K).toarray(), np.diag(md), eigvals_only=True)
    np.testing.assert_allclose(np.sort(r["eigs"]), w[:4], rtol=1e-9)


def test_zpjdrevcom_device_tight_binding(gpu):
    ia, ja, a = M.tight_binding3d(8)
    ops = DeviceOps(ia, ja, a, torch.complex128)
    r = gpu.zpjdrevcom((a.copy(), ja.copy(), ia.copy()), 4, ops.matvec, isearch=0, madspace=20, maxit=5000,
                       tol=1e-10, droptol=1e-3, icntl=(0, 0, 0, 0, 0), device=True)
    assert r["info"] == 0 and r["neig"] == 4
    w = np.linalg.eigvalsh(M.to_scipy_full(ia, ja, a).toarray())
    np.testing.assert_allclose(np.sort(r["eigs"]), w[:4], rtol=1e-9, atol=1e-12)


def test_device_ptr_without_pending_request(gpu):
    L = gpu.load()
    xd, st = C.c_void_p(), C.c_void_p()
    assert L.jdgpu_revcom_device_ptr(0, C.byref(xd), C.byref(st)) == -1
    assert L.jdgpu_revcom_device_ptr(1, C.byref(xd), C.byref(st)) == -1
