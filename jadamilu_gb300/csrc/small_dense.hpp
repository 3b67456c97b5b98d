// Small dense linear algebra on the host for the J x J projected problems of
// the Jacobi-Davidson loop (J <= MADSPACE, a few dozen at most).
//
// The reference calls LAPACK/BLAS for these (src/include/ilupackmacros.h:55-72,
// used at src/jd/JDaux.F:1651-1659, 2027-2031, 2430-2449, 3294-3331).  No
// LAPACK is linked; each operation is written from its definition: Hermitian
// eigenproblems by cyclic Jacobi, Cholesky, Householder QR, and the BLAS-2/3
// products on J x J data.  Column-major storage with a leading dimension, as
// in the reference workspace.  The N-length vector helpers (dotc, nrm2, axpy,
// gemv_*) are used by the CPU oracle only; the GPU library runs those on the
// device.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <numeric>
#include <limits>
#include <type_traits>
#include <vector>

namespace jdd {

using cplx = std::complex<double>;
inline double re(double x) { return x; }
inline double re(cplx x) { return x.real(); }
inline double cj(double x) { return x; }
inline cplx cj(cplx x) { return std::conj(x); }
inline float cj(float x) { return x; }
inline std::complex<float> cj(std::complex<float> x) { return std::conj(x); }
inline double ab(double x) { return std::fabs(x); }
inline double ab(cplx x) { return std::abs(x); }
inline double ab2(double x) { return x * x; }
inline double ab2(cplx x) { return std::norm(x); }

template <class T> T dotc(long n, const T* x, const T* y) {
  T s = T(0);
  for (long i = 0; i < n; ++i) s += cj(x[i]) * y[i];
  return s;
}
template <class T> double nrm2(long n, const T* x) {
  double s = 0;
  for (long i = 0; i < n; ++i) s += ab2(x[i]);
  return std::sqrt(s);
}
template <class T> void axpy(long n, T a, const T* x, T* y) {
  for (long i = 0; i < n; ++i) y[i] += a * x[i];
}
template <class T> void rscal(long n, double a, T* x) {
  for (long i = 0; i < n; ++i) x[i] *= a;
}
template <class T> void copyv(long n, const T* x, T* y) { std::memmove(y, x, sizeof(T) * n); }
template <class T> void fillv(long n, T v, T* y) {
  for (long i = 0; i < n; ++i) y[i] = v;
}
// y = alpha*A*x + beta*y, A n x m (lda)
template <class T> void gemv_n(long n, long m, T alpha, const T* A, long lda, const T* x, T beta, T* y) {
  for (long i = 0; i < n; ++i) y[i] = (beta == T(0)) ? T(0) : beta * y[i];
  for (long j = 0; j < m; ++j) {
    T t = alpha * x[j];
    const T* a = A + j * lda;
    for (long i = 0; i < n; ++i) y[i] += t * a[i];
  }
}
// y = alpha*A^H*x + beta*y, A n x m (lda)
template <class T> void gemv_c(long n, long m, T alpha, const T* A, long lda, const T* x, T beta, T* y) {
  for (long j = 0; j < m; ++j) {
    T s = dotc(n, A + j * lda, x);
    y[j] = alpha * s + ((beta == T(0)) ? T(0) : beta * y[j]);
  }
}
// upper triangle of a Hermitian J x J matrix (ld) times x
template <class T> void hemv_u(long J, const T* M, long ld, const T* x, T* y) {
  for (long i = 0; i < J; ++i) {
    T s = T(0);
    for (long k = 0; k < J; ++k) {
      T mik = (i <= k) ? M[i + k * ld] : cj(M[k + i * ld]);
      if (i == k) mik = T(re(mik));
      s += mik * x[k];
    }
    y[i] = s;
  }
}
// fill the lower triangle of a Hermitian matrix from its upper triangle
template <class T> void herm_full(long J, T* M, long ld) {
  for (long j = 0; j < J; ++j) {
    M[j + j * ld] = T(re(M[j + j * ld]));
    for (long i = j + 1; i < J; ++i) M[i + j * ld] = cj(M[j + i * ld]);
  }
}

// Cyclic Jacobi for a Hermitian J x J matrix (full storage, ld).  On exit w
// holds the eigenvalues in ascending order and A the orthonormal eigenvectors
// (columns).  Returns 0, or 1 if the sweeps did not converge.
template <class T> int heev(long J, T* A, long ld, double* w) {
  std::vector<T> a(J * J), v(J * J, T(0));
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) a[i + j * J] = A[i + j * ld];
  for (long i = 0; i < J; ++i) v[i + i * J] = T(1);
  int conv = 0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (long j = 0; j < J; ++j)
      for (long i = 0; i < J; ++i) {
        tot += ab2(a[i + j * J]);
        if (i != j) off += ab2(a[i + j * J]);
      }
    if (off <= 1e-34 * tot || off == 0) { conv = 1; break; }
    for (long p = 0; p < J - 1; ++p)
      for (long q = p + 1; q < J; ++q) {
        T apq = a[p + q * J];
        double g = ab(apq);
        if (g == 0) continue;
        double app = re(a[p + p * J]), aqq = re(a[q + q * J]);
        if (g < 1e-300) continue;
        T ph = apq / g;  // unit phase
        double tau = (aqq - app) / (2 * g);
        double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        double c = 1 / std::sqrt(1 + t * t), s = t * c;
        // unitary U acting on columns p,q: col_p' = c col_p - s conj(ph) col_q ; col_q' = s ph col_p + c col_q
        T up = T(-s) * cj(ph), uq = T(s) * ph;
        for (long k = 0; k < J; ++k) {  // A := A U
          T akp = a[k + p * J], akq = a[k + q * J];
          a[k + p * J] = c * akp + up * akq;
          a[k + q * J] = uq * akp + c * akq;
          T vkp = v[k + p * J], vkq = v[k + q * J];
          v[k + p * J] = c * vkp + up * vkq;
          v[k + q * J] = uq * vkp + c * vkq;
        }
        for (long k = 0; k < J; ++k) {  // A := U^H A
          T apk = a[p + k * J], aqk = a[q + k * J];
          a[p + k * J] = c * apk + cj(up) * aqk;
          a[q + k * J] = cj(uq) * apk + c * aqk;
        }
        a[p + q * J] = T(0);
        a[q + p * J] = T(0);
        a[p + p * J] = T(re(a[p + p * J]));
        a[q + q * J] = T(re(a[q + q * J]));
      }
  }
  std::vector<long> idx(J);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](long x, long y) { return re(a[x + x * J]) < re(a[y + y * J]); });
  for (long k = 0; k < J; ++k) {
    w[k] = re(a[idx[k] + idx[k] * J]);
    for (long i = 0; i < J; ++i) A[i + k * ld] = v[i + idx[k] * J];
  }
  return conv ? 0 : 1;
}

// Cholesky B = L L^H in place (lower, ld).  Returns 0 or the failing column+1.
template <class T> int potrf_l(long J, T* B, long ld) {
  for (long j = 0; j < J; ++j) {
    double d = re(B[j + j * ld]);
    for (long k = 0; k < j; ++k) d -= ab2(B[j + k * ld]);
    if (!(d > 0)) return (int)j + 1;
    d = std::sqrt(d);
    B[j + j * ld] = T(d);
    for (long i = j + 1; i < J; ++i) {
      T s = B[i + j * ld];
      for (long k = 0; k < j; ++k) s -= B[i + k * ld] * cj(B[j + k * ld]);
      B[i + j * ld] = s / d;
    }
  }
  return 0;
}

// Generalized Hermitian-definite problem A y = lambda B y (type 1), A and B
// given by their upper triangles.  Eigenvalues ascending in w, B-orthonormal
// eigenvectors in A; B is overwritten by its Cholesky factor.
template <class T> int hegv(long J, T* A, long lda, T* B, long ldb, double* w) {
  herm_full(J, B, ldb);
  int info = potrf_l(J, B, ldb);
  if (info) return J + info;
  herm_full(J, A, lda);
  // C = L^{-1} A L^{-H}
  std::vector<T> C(J * J);
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) C[i + j * J] = A[i + j * lda];
  for (long j = 0; j < J; ++j)  // solve L X = A (columns)
    for (long i = 0; i < J; ++i) {
      T s = C[i + j * J];
      for (long k = 0; k < i; ++k) s -= B[i + k * ldb] * C[k + j * J];
      C[i + j * J] = s / B[i + i * ldb];
    }
  for (long i = 0; i < J; ++i)  // solve X L^H = C (rows): C := C L^{-H}
    for (long j = 0; j < J; ++j) {
      T s = C[i + j * J];
      for (long k = 0; k < j; ++k) s -= C[i + k * J] * cj(B[j + k * ldb]);
      C[i + j * J] = s / B[j + j * ldb];
    }
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) C[i + j * J] = 0.5 * (C[i + j * J] + cj(C[j + i * J]));
  info = heev(J, C.data(), J, w);
  // y = L^{-H} z
  for (long j = 0; j < J; ++j)
    for (long i = J - 1; i >= 0; --i) {
      T s = C[i + j * J];
      for (long k = i + 1; k < J; ++k) s -= cj(B[k + i * ldb]) * C[k + j * J];
      C[i + j * J] = s / B[i + i * ldb];
    }
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) A[i + j * lda] = C[i + j * J];
  return info;
}

// Solve N X = M for the J x J Hermitian positive definite N (upper triangle
// given) and J right-hand sides M (J x J, ld); M is overwritten by X and N by
// its Cholesky factor.  Returns 0 or the failing column+1 (POSV semantics).
template <class T> int posv_u(long J, T* N, long ldn, T* M, long ldm) {
  herm_full(J, N, ldn);
  int info = potrf_l(J, N, ldn);
  if (info) return info;
  for (long c = 0; c < J; ++c) {
    T* x = M + c * ldm;
    for (long i = 0; i < J; ++i) {  // L y = m
      T s = x[i];
      for (long k = 0; k < i; ++k) s -= N[i + k * ldn] * x[k];
      x[i] = s / N[i + i * ldn];
    }
    for (long i = J - 1; i >= 0; --i) {  // L^H x = y
      T s = x[i];
      for (long k = i + 1; k < J; ++k) s -= cj(N[k + i * ldn]) * x[k];
      x[i] = s / N[i + i * ldn];
    }
  }
  return 0;
}

// Eigenvalues and right eigenvectors of a general J x J matrix A (ld), in
// complex arithmetic: Householder reduction to Hessenberg form, single-shift
// QR sweeps (Wilkinson shift from the trailing 2 x 2 block, an exceptional
// shift after 10 sweeps without deflation) to the triangular Schur form
// T = Q^H A Q, eigenvectors of T by back substitution, back to A by Q.
// Each eigenvector is scaled to unit 2-norm with its largest component real
// (the GEEV convention).  wr receives the real parts of the eigenvalues
// (unsorted); V (ld) the eigenvectors (real parts for real T).  Returns 0, or
// 1 when the QR sweeps do not converge.
template <class T> int geev_right(long J, const T* A, long lda, double* wr, T* V, long ldv) {
  using Z = std::complex<double>;
  std::vector<Z> H((size_t)J * J), Q((size_t)J * J, Z(0));
  auto h = [&](long i, long j) -> Z& { return H[i + j * J]; };
  auto q = [&](long i, long j) -> Z& { return Q[i + j * J]; };
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) h(i, j) = Z(A[i + j * lda]);
  for (long i = 0; i < J; ++i) q(i, i) = Z(1);
  // Hessenberg reduction: reflector P = I - 2 v v^H / (v^H v) zeroes column k below k+1
  for (long k = 0; k + 2 < J; ++k) {
    double nrm = 0;
    for (long i = k + 1; i < J; ++i) nrm += std::norm(h(i, k));
    nrm = std::sqrt(nrm);
    if (nrm == 0) continue;
    std::vector<Z> v(J, Z(0));
    const Z a = h(k + 1, k);
    const Z ph = std::abs(a) > 0 ? a / std::abs(a) : Z(1);
    v[k + 1] = a + ph * nrm;
    for (long i = k + 2; i < J; ++i) v[i] = h(i, k);
    double vv = 0;
    for (long i = k + 1; i < J; ++i) vv += std::norm(v[i]);
    if (vv == 0) continue;
    for (long j = 0; j < J; ++j) {  // H := P H
      Z s = 0;
      for (long i = k + 1; i < J; ++i) s += std::conj(v[i]) * h(i, j);
      s *= 2.0 / vv;
      for (long i = k + 1; i < J; ++i) h(i, j) -= v[i] * s;
    }
    for (long i = 0; i < J; ++i) {  // H := H P, Q := Q P
      Z s = 0, t = 0;
      for (long j = k + 1; j < J; ++j) {
        s += h(i, j) * v[j];
        t += q(i, j) * v[j];
      }
      s *= 2.0 / vv;
      t *= 2.0 / vv;
      for (long j = k + 1; j < J; ++j) {
        h(i, j) -= s * std::conj(v[j]);
        q(i, j) -= t * std::conj(v[j]);
      }
    }
    for (long i = k + 2; i < J; ++i) h(i, k) = 0;
  }
  double anorm = 0;
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < J; ++i) anorm = std::max(anorm, std::abs(h(i, j)));
  const double eps = std::numeric_limits<double>::epsilon();
  // shifted QR on the active window [lo, hi]
  long hi = J - 1;
  int stall = 0, total = 0;
  while (hi > 0) {
    long lo = hi;
    while (lo > 0) {
      const double sub = std::abs(h(lo, lo - 1));
      const double dia = std::abs(h(lo, lo)) + std::abs(h(lo - 1, lo - 1));
      if (sub <= eps * (dia > 0 ? dia : anorm)) {
        h(lo, lo - 1) = 0;
        break;
      }
      --lo;
    }
    if (lo == hi) {  // one eigenvalue deflated
      --hi;
      stall = 0;
      continue;
    }
    if (++total > 60 * J) return 1;
    // Wilkinson shift: eigenvalue of the trailing 2 x 2 block closer to h(hi, hi)
    Z mu;
    if (++stall % 11 == 10) {
      mu = h(hi, hi) + Z(std::abs(h(hi, hi - 1)) * 0.75, 0);
    } else {
      const Z a = h(hi - 1, hi - 1), b = h(hi - 1, hi), c = h(hi, hi - 1), d = h(hi, hi);
      const Z tr = a + d, det = a * d - b * c;
      const Z disc = std::sqrt(tr * tr * 0.25 - det);
      const Z l1 = tr * 0.5 + disc, l2 = tr * 0.5 - disc;
      mu = std::abs(l1 - d) < std::abs(l2 - d) ? l1 : l2;
    }
    // one QR sweep on H(lo:hi, lo:hi) - mu I by Givens rotations (bulge chase)
    Z x = h(lo, lo) - mu, y = h(lo + 1, lo);
    for (long k = lo; k < hi; ++k) {
      const double r = std::sqrt(std::norm(x) + std::norm(y));
      const Z cs = r > 0 ? x / r : Z(1), sn = r > 0 ? y / r : Z(0);
      // G = [conj(cs) conj(sn); -sn cs] applied to rows k, k+1 (columns from max(lo, k-1))
      for (long j = std::max(lo, k - 1); j < J; ++j) {
        const Z u = h(k, j), w = h(k + 1, j);
        h(k, j) = std::conj(cs) * u + std::conj(sn) * w;
        h(k + 1, j) = -sn * u + cs * w;
      }
      // columns k, k+1 with G^H (rows up to min(hi, k+2)); accumulate Q
      for (long i = 0; i <= std::min(hi, k + 2); ++i) {
        const Z u = h(i, k), w = h(i, k + 1);
        h(i, k) = u * cs + w * sn;
        h(i, k + 1) = -u * std::conj(sn) + w * std::conj(cs);
      }
      for (long i = 0; i < J; ++i) {
        const Z u = q(i, k), w = q(i, k + 1);
        q(i, k) = u * cs + w * sn;
        q(i, k + 1) = -u * std::conj(sn) + w * std::conj(cs);
      }
      if (k + 1 < hi) {
        x = h(k + 1, k);
        y = h(k + 2, k);
      }
    }
  }
  // eigenvectors of the triangular T = H, then V = Q Z
  std::vector<Z> zv(J), col(J);
  for (long k = 0; k < J; ++k) {
    const Z lam = h(k, k);
    std::fill(zv.begin(), zv.end(), Z(0));
    zv[k] = Z(1);
    for (long i = k - 1; i >= 0; --i) {
      Z s = 0;
      for (long j = i + 1; j <= k; ++j) s += h(i, j) * zv[j];
      Z den = h(i, i) - lam;
      if (std::abs(den) < eps * anorm) den = Z(eps * std::max(anorm, 1e-300), 0);
      zv[i] = -s / den;
    }
    double nrm = 0;
    long imax = 0;
    for (long i = 0; i < J; ++i) {
      Z s = 0;
      for (long j = 0; j <= k; ++j) s += q(i, j) * zv[j];
      col[i] = s;
      nrm += std::norm(s);
      if (std::abs(s) > std::abs(col[imax])) imax = i;
    }
    nrm = std::sqrt(nrm);
    const Z ph = std::abs(col[imax]) > 0 ? std::conj(col[imax]) / std::abs(col[imax]) : Z(1);
    for (long i = 0; i < J; ++i) {
      const Z c = col[i] * ph / nrm;
      if constexpr (std::is_same<T, double>::value) V[i + k * ldv] = c.real();
      else V[i + k * ldv] = T(c);
    }
    wr[k] = lam.real();
  }
  return 0;
}

// Householder QR of the K x J matrix U (ld); returns the explicit K x K
// unitary factor Q (column-major, K) whose first J columns span U.
template <class T> void householder_q(long K, long J, const T* U, long ld, std::vector<T>& Q) {
  std::vector<T> a(K * J);
  for (long j = 0; j < J; ++j)
    for (long i = 0; i < K; ++i) a[i + j * K] = U[i + j * ld];
  std::vector<std::vector<T>> vs;
  std::vector<T> taus;
  for (long j = 0; j < J && j < K; ++j) {
    double xn = 0;
    for (long i = j; i < K; ++i) xn += ab2(a[i + j * K]);
    xn = std::sqrt(xn);
    std::vector<T> v(K, T(0));
    T tau = T(0);
    if (xn > 0) {
      T alpha = a[j + j * K];
      T beta = (ab(alpha) > 0 ? -alpha / ab(alpha) : T(-1)) * xn;  // beta = -phase(alpha)*|x|
      for (long i = j; i < K; ++i) v[i] = a[i + j * K];
      v[j] -= beta;
      double vn2 = 0;
      for (long i = j; i < K; ++i) vn2 += ab2(v[i]);
      if (vn2 > 0) {
        tau = T(2.0 / vn2);
        for (long c = j; c < J; ++c) {  // a := (I - tau v v^H) a
          T s = T(0);
          for (long i = j; i < K; ++i) s += cj(v[i]) * a[i + c * K];
          s *= tau;
          for (long i = j; i < K; ++i) a[i + c * K] -= s * v[i];
        }
      }
    }
    vs.push_back(v);
    taus.push_back(tau);
  }
  Q.assign(K * K, T(0));
  for (long i = 0; i < K; ++i) Q[i + i * K] = T(1);
  // Q = H_1 H_2 ... H_J applied to I from the left in reverse order
  for (long j = (long)vs.size() - 1; j >= 0; --j) {
    const std::vector<T>& v = vs[j];
    for (long c = 0; c < K; ++c) {
      T s = T(0);
      for (long i = j; i < K; ++i) s += cj(v[i]) * Q[i + c * K];
      s *= taus[j];
      for (long i = j; i < K; ++i) Q[i + c * K] -= s * v[i];
    }
  }
}

// X (n x K, ld n) := X * Q (Q: K x K); only the first `keep` columns are formed.
template <class T> void right_mult(long n, long K, long keep, T* X, const std::vector<T>& Q) {
  std::vector<T> row(K), out(keep);
  for (long i = 0; i < n; ++i) {
    for (long k = 0; k < K; ++k) row[k] = X[i + k * n];
    for (long c = 0; c < keep; ++c) {
      T s = T(0);
      for (long k = 0; k < K; ++k) s += row[k] * Q[k + c * K];
      out[c] = s;
    }
    for (long c = 0; c < keep; ++c) X[i + c * n] = out[c];
  }
}

// Index sort: idx[k] (0-based) such that key[idx[0]] <= key[idx[1]] <= ...
inline void sort_index(long n, const double* key, long* idx) {
  for (long i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx, idx + n, [&](long a, long b) { return key[a] < key[b]; });
}

}  // namespace jdd
