// Jacobi-Davidson core on device vectors (host control, sm_103a kernels).
//
// Same algorithm as the reference's JDRVCOM/LSOLREVCOM/STOPTEST/REPGS/
// SOLPROJEP/SHRINK/SORTEV (src/jd/JDaux.F:1391-3358).  Every N-length vector
// lives on the GPU in `dX`, a device copy of the caller's workspace X with the
// reference layout (JDaux.F:1534-1567), so reverse-communication offsets
// (NDX1/NDX2/NDX3) and the eigenvector output keep their meaning.  The J x J
// projected matrices and the small coefficient vectors stay in the caller's
// host X at the same offsets.  Scalars that steer the control flow (norms,
// inner products) are read back with one stream synchronisation each.
#pragma once
#include <cfloat>
#include <complex>
#include <functional>
#include <vector>

#include "kernels.cuh"
#include "small_dense.hpp"

namespace jdg {

template <class T> struct HostOf { using type = double; };
template <> struct HostOf<zc> { using type = std::complex<double>; };
inline double hre(double x) { return x; }
inline double hre(std::complex<double> x) { return x.real(); }
inline double habs(double x) { return std::fabs(x); }
inline double habs(std::complex<double> x) { return std::abs(x); }
inline double tod(double x) { return x; }
inline zc todev(std::complex<double> x) { return zc(x.real(), x.imag()); }
inline double todev(double x) { return x; }

// values shared with the preconditioner-aware driver (COMMON /JDRVCOMJD/)
struct JdState {
  double timeilu = 0, rinit = 0, rcurr = 0, rcum = 0, shift1 = 0;
  bool flagcg = false;
};

// Device workspace of one solve.
template <class T> struct Workspace {
  cudaStream_t st = nullptr;
  long N = 0, LX = 0, cap_x = 0, cap_tmp = 0, cap_part = 0;
  T* dX = nullptr;     // device copy of X
  T* dsm = nullptr;    // small device results (<= 512)
  T* hsm = nullptr;    // pinned host mirror
  T* dpart = nullptr;  // reduction partials
  T* dtmp = nullptr;   // N x 32 scratch for restarts
  bool own_stream = false;
  void set_stream(cudaStream_t s) {
    if (own_stream && st) cudaStreamDestroy(st);
    st = s;
    own_stream = false;
  }
  void ensure(long n, long lx) {
    if (!st) {
      CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      own_stream = true;
    }
    if (!dsm) {
      CK(cudaMalloc(&dsm, sizeof(T) * 512));
      CK(cudaMallocHost(&hsm, sizeof(T) * 512));
    }
    if (lx > cap_x) {
      if (dX) CK(cudaFree(dX));
      CK(cudaMalloc(&dX, sizeof(T) * lx));
      cap_x = lx;
    }
    long need_tmp = n * 32;
    if (need_tmp > cap_tmp) {
      if (dtmp) CK(cudaFree(dtmp));
      CK(cudaMalloc(&dtmp, sizeof(T) * need_tmp));
      cap_tmp = need_tmp;
    }
    long need_part = k::mdot_partial_size(n, 128);
    if (need_part > cap_part) {
      if (dpart) CK(cudaFree(dpart));
      CK(cudaMalloc(&dpart, sizeof(T) * need_part));
      CK(cudaMemset(dpart, 0, sizeof(T) * need_part));  // the reduction's arrival counter starts at zero
      cap_part = need_part;
    }
    N = n;
    LX = lx;
  }
  // frees everything (the workspace of a batch worker ends with its thread)
  void release() {
    if (dX) cudaFree(dX);
    if (dsm) cudaFree(dsm);
    if (hsm) cudaFreeHost(hsm);
    if (dpart) cudaFree(dpart);
    if (dtmp) cudaFree(dtmp);
    if (own_stream && st) cudaStreamDestroy(st);
    dX = dsm = hsm = dpart = dtmp = nullptr;
    st = nullptr;
    own_stream = false;
    cap_x = cap_tmp = cap_part = 0;
  }
  ~Workspace() {}
};

template <class T> struct StopStateD {
  int istag = 0, istt = 0;
  bool posdef = false, toupdate = false;
  double g0 = 0, gs = 0, gtrs = 0, gkmin = 0, bk = 0, beta = 0, tn = 0, un2 = -1, gkm1 = 0, alp = 1;
  typename HostOf<T>::type bkgep = 0, bubt = 0;
};

struct Lcg48d {
  unsigned long long s = 0x1234ABCD330EULL;
  double next() {
    s = (s * 0x5DEECE66DULL + 0xB) & ((1ULL << 48) - 1);
    return ((double)(s >> 5) + 0.5) / (double)(1ULL << 43);
  }
};

template <class T> struct DevJd {
  using H = typename HostOf<T>::type;
  Workspace<T>* W = nullptr;
  JdState* sh = nullptr;
  H* hX = nullptr;  // caller's X (small J x J data live here)
  // which: 1 = A x (and B x for GEP), 3 = A x, 4 = B x; offsets into X
  std::function<void(int, long, long, long)> matvec;
  std::function<void(long, long)> precond;  // (rhs, sol)
  // optional y = A x + a x in one pass (built-in matrix, no B)
  std::function<void(long, long, H)> matvec_shift;
  std::function<void(int, int, int, double, double)> on_step;  // progress printer (may be empty)
  StopStateD<T> st;
  Lcg48d rng;
  double alpha_cg = 0;
  int istag = 0;
  long launches = 0;
  // The operators are the library's own stream-ordered kernels (no host
  // round trip inside matvec/precond): the inner iteration may then keep its
  // scalars on the device and read them back once per iteration.
  bool device_ops = false;
  static constexpr int kScal = 500;  // dsm slots of the inner-iteration scalars

  T* D(long off) { return W->dX + off; }
  cudaStream_t S() { return W->st; }
  void sync() { CK(cudaStreamSynchronize(S())); }

  // ---- device primitives on X offsets ----
  double nrm2(long n, long x) {
    k::mdot<T>(n, 1, D(x), n, D(x), W->dsm, W->dpart, S());
    CK(cudaMemcpyAsync(W->hsm, W->dsm, sizeof(T), cudaMemcpyDeviceToHost, S()));
    sync();
    return std::sqrt(rl(W->hsm[0]));
  }
  H dot(long n, long x, long y) {
    k::mdot<T>(n, 1, D(x), n, D(y), W->dsm, W->dpart, S());
    CK(cudaMemcpyAsync(W->hsm, W->dsm, sizeof(T), cudaMemcpyDeviceToHost, S()));
    sync();
    return reinterpret_cast<H*>(W->hsm)[0];
  }
  // out_host[c] = X(V + c*ldv)^H X(w), c < k
  void gemvc(long n, int kc, long V, long ldv, long w, H* out_host) {
    if (kc <= 0) return;
    for (int c0 = 0; c0 < kc; c0 += 128) {
      int kk = std::min(128, kc - c0);
      k::mdot<T>(n, kk, D(V + (long)c0 * ldv), ldv, D(w), W->dsm, W->dpart, S());
      CK(cudaMemcpyAsync(W->hsm, W->dsm, sizeof(T) * kk, cudaMemcpyDeviceToHost, S()));
      sync();
      for (int c = 0; c < kk; ++c) out_host[c0 + c] = reinterpret_cast<H*>(W->hsm)[c];
    }
  }
  // X(w) = beta X(w) + alpha X(V) y, y on the host
  void gemvn(long n, int kc, H alpha, long V, long ldv, const H* y, H beta, long w) {
    std::vector<T> yd(std::max(kc, 1));
    for (int c = 0; c < kc; ++c) yd[c] = todev(y[c]);
    for (int c0 = 0; c0 < std::max(kc, 1); c0 += 64) {
      int kk = std::min(64, kc - c0);
      H b = (c0 == 0) ? beta : H(1);
      k::gemv_val<T>(n, std::max(kk, 0), todev(alpha), D(V + (long)c0 * ldv), ldv, yd.data() + c0, todev(b), D(w), S());
      if (kc <= 0) break;
    }
  }
  void axpy(long n, H a, long x, long y) { k::axpy<T>(n, todev(a), D(x), D(y), S()); }
  // classical Gram-Schmidt of REPGS (gam < 0) with the coefficients left in
  // device memory at cdev
  void cgs_dev(long N, long V, long BV, long JV, long w, T* cdev) {
    k::mdot<T>(N, (int)JV, D(BV), N, D(w), cdev, W->dpart, S());
    k::gemv_dev<T>(N, (int)JV, T(-1), D(V), N, cdev, T(1), D(w), S());
  }
  void scal(long n, double a, long x) { k::scal<T>(n, a, D(x), S()); }
  void copy(long n, long x, long y) {
    if (n > 0 && x != y) CK(cudaMemcpyAsync(D(y), D(x), sizeof(T) * n, cudaMemcpyDeviceToDevice, S()));
  }
  void fill(long n, H v, long x) { k::fill<T>(n, todev(v), D(x), S()); }

  // REPGS on device vectors; y (coefficients and final norm) on the host
  void repgs(long N, long V, long BV, long JV, long w, H* y, double epsm, int gam) {
    bool nrnd = true;
    if (JV <= 0) return;
    if (gam < 0) {
      // classical Gram-Schmidt, coefficients stay on the device
      if (JV > 64) throw std::runtime_error("projection against more than 64 vectors");
      k::mdot<T>(N, (int)JV, D(BV), N, D(w), W->dsm, W->dpart, S());
      k::gemv_dev<T>(N, (int)JV, T(-1), D(V), N, W->dsm, T(1), D(w), S());
      if (y) {
        CK(cudaMemcpyAsync(W->hsm, W->dsm, sizeof(T) * JV, cudaMemcpyDeviceToHost, S()));
        sync();
        for (long c = 0; c < JV; ++c) y[c] = reinterpret_cast<H*>(W->hsm)[c];
      }
      return;
    }
    for (;;) {
      double nrn = nrm2(N, w), nr = epsm * nrn, nro;
      if (nrnd)
        for (long c = 0; c < JV; ++c) y[c] = H(0);
      bool small = false;
      do {
        nro = nrn;
        gemvc(N, (int)JV, BV, N, w, y + JV);
        gemvn(N, (int)JV, H(-1), V, N, y + JV, H(1), w);
        nrn = nrm2(N, w);
        if (nrnd)
          for (long c = 0; c < JV; ++c) y[c] += y[JV + c];
        if (nrn <= nr) { small = true; break; }
      } while (nrn < 0.5 * nro);
      if (!small) { y[JV] = H(nrn); return; }
      if (gam == 1) {
        if (JV < N) {
          std::vector<T> r(N);
          for (long i = 0; i < N; ++i) r[i] = T(rng.next());
          CK(cudaMemcpyAsync(D(w), r.data(), sizeof(T) * N, cudaMemcpyHostToDevice, S()));
          sync();
          nrnd = false;
          continue;
        }
      } else {
        fill(N, H(0), w);
        y[JV] = H(0);
      }
      return;
    }
  }

  // SORTEV on host arrays (small) or device columns (eigenvectors)
  void sort_index_key(long J, const double* eigs, int it, double sigma, std::vector<long>& iw) {
    std::vector<double> key(J);
    for (long i = 0; i < J; ++i) {
      if (it == 2 || it == -2) key[i] = -std::fabs(eigs[i] - sigma);
      else if (it == 4 || it == -4) key[i] = eigs[i];
      else key[i] = -eigs[i];
    }
    iw.resize(J);
    jdd::sort_index(J, key.data(), iw.data());
    if (it == -2) {
      long last = iw[J - 1];
      for (long i = J - 1; i > 0; --i) iw[i] = iw[i - 1];
      iw[0] = last;
    }
  }
  void sortev_host(long J, H* V, long ldv, double* eigs, int it) {
    if (J <= 1) return;
    std::vector<long> iw;
    sort_index_key(J, eigs, it, 0.0, iw);
    std::vector<H> tv(J * J);
    for (long c = 0; c < J; ++c)
      for (long r = 0; r < J; ++r) tv[r + c * J] = V[r + iw[c] * ldv];
    for (long c = 0; c < J; ++c)
      for (long r = 0; r < J; ++r) V[r + c * ldv] = tv[r + c * J];
    std::vector<double> te(J);
    for (long c = 0; c < J; ++c) te[c] = eigs[iw[c]];
    for (long c = 0; c < J; ++c) eigs[c] = te[c];
  }
  void sortev_dev(long N, long J, long V, long V2, double* eigs, double* r, int it, double sigma) {
    if (J <= 1) return;
    std::vector<long> iw;
    sort_index_key(J, eigs, it, sigma, iw);
    auto permute = [&](long base) {
      for (long c = 0; c < J; ++c)
        CK(cudaMemcpyAsync(W->dtmp + c * N, D(base + iw[c] * N), sizeof(T) * N, cudaMemcpyDeviceToDevice, S()));
      CK(cudaMemcpyAsync(D(base), W->dtmp, sizeof(T) * N * J, cudaMemcpyDeviceToDevice, S()));
    };
    if (J > 32) throw std::runtime_error("sortev: more than 32 vectors");
    permute(V);
    if (it == -4) permute(V2);
    std::vector<double> te(J);
    for (long c = 0; c < J; ++c) te[c] = eigs[iw[c]];
    for (long c = 0; c < J; ++c) eigs[c] = te[c];
    if (it == 4 || it == -4) {
      for (long c = 0; c < J; ++c) te[c] = r[iw[c]];
      for (long c = 0; c < J; ++c) r[c] = te[c];
    }
  }
  // SOLPROJEP (JDaux.F:3271-3358); the generalized harmonic case solves
  // NN X = MM (POSV) and takes the right eigenvectors of X (GEEV).
  void solprojep(long J, H* MM, H* NN, long ld, double& theta, double& theta2, double* w, int is, int& info, bool gep) {
    if (is == 2 || is == -2) {
      if (gep) {
        info = jdd::posv_u(J, NN, ld, MM, ld);
        if (info) return;
        jdd::copyv(ld * ld, MM, NN);
        info = jdd::geev_right(J, NN, ld, w, MM, ld);
        if (info) return;
        sortev_host(J, MM, ld, w, is);
        theta2 = w[1];
        return;
      }
      info = jdd::hegv(J, MM, ld, NN, ld, w);
      if (info) return;
      sortev_host(J, MM, ld, w, is);
      theta2 = w[1];
      return;
    }
    jdd::herm_full(J, MM, ld);
    info = jdd::heev(J, MM, ld, w);
    if (info) return;
    if (is == 3) {
      for (long i = 0; i < J; ++i) NN[i] = H(w[i]);
    } else {
      theta = w[0];
      theta2 = w[1];
    }
  }
  void shrink(long N, long J, long K, const H* U, long ldu, long V, long Wv, long BV, H* MM, H* NN, long ld,
              int iserch, bool gep) {
    if (K > 32) throw std::runtime_error("shrink: search space above 32");
    std::vector<H> Q;
    jdd::householder_q(K, J, U, ldu, Q);
    std::vector<T> qd(K * K);
    for (long i = 0; i < K * K; ++i) qd[i] = todev(Q[i]);
    auto apply = [&](long base) {
      k::rmult<T>(N, (int)K, (int)J, D(base), N, qd.data(), W->dtmp, S());
      CK(cudaMemcpyAsync(D(base), W->dtmp, sizeof(T) * N * J, cudaMemcpyDeviceToDevice, S()));
    };
    apply(V);
    apply(Wv);
    if (gep) apply(BV);
    auto congr = [&](H* M, bool herm) {
      if (herm)
        for (long i = 1; i < K; ++i)
          for (long j = 0; j < i; ++j) M[i + j * ld] = jdd::cj(M[j + i * ld]);
      std::vector<H> tmp(K * K), out(K * K);
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) {
          H s = H(0);
          for (long kk = 0; kk < K; ++kk) s += M[i + kk * ld] * Q[kk + j * K];
          tmp[i + j * K] = s;
        }
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) {
          H s = H(0);
          for (long kk = 0; kk < K; ++kk) s += jdd::cj(Q[kk + i * K]) * tmp[kk + j * K];
          out[i + j * K] = s;
        }
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) M[i + j * ld] = out[i + j * K];
    };
    congr(MM, iserch != 2 || !gep);
    if (iserch == 2) congr(NN, true);
  }
  void stoptest(long N, long x, long bt, long bu, double tol, double& rk, double nbu, double& alprho, double& gk,
                H pcad, H pcr, double& theta, double eta, int& info, double trs, bool gep);
  void run(long N, double* EIGS, double* RES, int LX, int& NEIG, double SIGMA, int ISEARCH, int NINIT, int MADSPACE,
           int& ITER, double TOL, int& INFO, double& GAP, bool GEP);
};

}  // namespace jdg
