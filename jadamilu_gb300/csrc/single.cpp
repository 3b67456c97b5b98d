// Single-precision drivers: SPJD, SPJD_GEP, SPJDREVCOM, SPJDREVCOM_GEP,
// SJDREVCOM, SJDREVCOM_GEP, SPJDCLEANUP and the COMPLEX set CPJD ...
// CPJDCLEANUP (reference Doc/SPJD_prototypes.f:3-798 and
// Doc/CPJD_prototypes.f:3-798; the reference compiles them from
// src/jd/PJD.F and JDaux.F with _SINGLE_REAL_ / _SINGLE_COMPLEX_,
// src/include/ilupackmacros.h:379-400 and 740-760).
//
// Same argument lists and protocol as the double drivers, with REAL
// (COMPLEX) values.  Each call widens the caller's values to double, runs the
// double-precision GPU driver on the widened copies and rounds what it wrote
// back into the caller's arrays; the iteration itself therefore runs in
// double precision.  A reverse-communication solve keeps its widened copies
// between calls and converts only the request vectors: before returning,
// the input of the request (X(NDX1), or X(NDX2) for a preconditioner solve)
// is rounded into the caller's X; on re-entry the caller's results
// (X(NDX2) and, for _GEP, X(NDX3); X(NDX1) for a preconditioner solve) are
// widened back.  The single drivers share the state of the double ones: a
// reverse-communication solve of SPJDREVCOM and one of DPJDREVCOM (CPJD... and
// ZPJD...) cannot be in flight together.
#include <complex>
#include <vector>

#include "../../include/jadamilu_gb300.h"

// In the 64-bit-integer library this unit is compiled a second time
// (JDG_ILP64_INNER): its drivers take the internal names of the 32-bit
// ones, call the 32-bit double drivers, and ilp64.cpp puts the 64-bit
// wrappers in front of them.
#ifdef JDG_ILP64_INNER
#define JDG_S(name) jdg_i32_##name
extern "C" {
void jdg_i32_dpjd_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*,
                   double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_dpjd_gep_(int*, double*, int*, int*, double*, int*, int*, double*, double*, double*, int*, int*, double*,
                       int*, int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_dpjdrevcom_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*,
                         int*, double*, double*, double*, double*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_dpjdrevcom_gep_(int*, double*, int*, int*, double*, int*, int*, double*, double*, double*, int*, int*,
                             double*, int*, int*, int*, int*, double*, double*, double*, double*, int*, int*, int*,
                             int*, int*, int*, int*, double*);
void jdg_i32_djdrevcom_(int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*, double*, int*,
                        int*, int*, int*, int*, double*);
void jdg_i32_djdrevcom_gep_(int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*, double*,
                            int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_dpjdcleanup_(void);
void jdg_i32_zpjd_(int*, jdg_zcomplex*, int*, int*, double*, double*, jdg_zcomplex*, int*, int*, double*, int*, int*,
                   int*, int*, double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_zpjd_gep_(int*, jdg_zcomplex*, int*, int*, jdg_zcomplex*, int*, int*, double*, double*, jdg_zcomplex*,
                       int*, int*, double*, int*, int*, int*, int*, double*, double*, double*, double*, int*, int*,
                       int*, double*);
void jdg_i32_zpjdrevcom_(int*, jdg_zcomplex*, int*, int*, double*, double*, jdg_zcomplex*, int*, int*, double*, int*,
                         int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, int*, int*, int*,
                         double*);
void jdg_i32_zpjdrevcom_gep_(int*, jdg_zcomplex*, int*, int*, jdg_zcomplex*, int*, int*, double*, double*,
                             jdg_zcomplex*, int*, int*, double*, int*, int*, int*, int*, double*, double*, double*,
                             double*, int*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_zjdrevcom_(int*, double*, double*, jdg_zcomplex*, int*, int*, double*, int*, int*, int*, int*, double*,
                        int*, int*, int*, int*, int*, double*);
void jdg_i32_zjdrevcom_gep_(int*, double*, double*, jdg_zcomplex*, int*, int*, double*, int*, int*, int*, int*,
                            double*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_zpjdcleanup_(void);
}
#define JDG_SAPI
#else
#define JDG_S(name) name
#define JDG_SAPI JDG_API
#endif

namespace {

using cf = std::complex<float>;
using zd = std::complex<double>;

template <class S> struct Wide;
template <> struct Wide<float> { using type = double; };
template <> struct Wide<cf> { using type = zd; };

template <class S, class D> void widen(const S* s, D* d, long n) {
  for (long i = 0; i < n; ++i) d[i] = D(s[i]);
}
inline void narrow(const double* d, float* s, long n) {
  for (long i = 0; i < n; ++i) s[i] = (float)d[i];
}
inline void narrow(const zd* d, cf* s, long n) {
  for (long i = 0; i < n; ++i) s[i] = cf((float)d[i].real(), (float)d[i].imag());
}

// Widened copies of one solve's arrays and scalars.
template <class S> struct Copies {
  using D = typename Wide<S>::type;
  std::vector<D> a, b, x;
  std::vector<double> eigs, res;
  double sigma = 0, tol = 0, shift = 0, droptol = 0, mem = 0, gap = 0;
  int neig_in = 0, lx = 0, n = 0;
  long nnz_a = 0, nnz_b = 0;
  bool diag_only = false;  // JA(1) < 0: A (and B) hold the N diagonal values, IA/IB/JB unreferenced
  int ijob = 0, ndx1 = 0, ndx2 = 0, ndx3 = 0;  // the request last handed to the caller

  void load(int N, const S* A, const int* JA, const int* IA, const S* B, const int* IB, const float* EIGS,
            const float* RES, const S* X, int LX, int NEIG, const float* SIGMA, const float* TOL,
            const float* SHIFT, const float* DROPTOL, const float* MEM, const float* GAP) {
    n = N;
    lx = LX;
    neig_in = NEIG;
    // diagonal preconditioning (PJD.F:309-317, 626-634): the reference reads
    // A(1..N) (and B(1..N)) only and leaves A, JA, IA, B, JB, IB unchanged
    diag_only = A && JA && JA[0] < 0;
    if (diag_only) {
      nnz_a = N;
      nnz_b = B ? N : 0;
    } else {
      nnz_a = A ? (long)IA[N] - IA[0] : 0;
      nnz_b = B ? (long)IB[N] - IB[0] : 0;
    }
    a.resize(nnz_a);
    if (A) widen(A, a.data(), nnz_a);
    b.resize(nnz_b);
    if (B) widen(B, b.data(), nnz_b);
    x.resize(LX > 0 ? LX : 0);
    widen(X, x.data(), (long)x.size());
    eigs.assign(NEIG > 0 ? NEIG : 0, 0.0);
    res.assign(eigs.size(), 0.0);
    for (size_t i = 0; i < eigs.size(); ++i) {
      eigs[i] = EIGS[i];
      res[i] = RES[i];
    }
    sigma = *SIGMA;
    tol = *TOL;
    shift = SHIFT ? *SHIFT : 0.0;
    droptol = DROPTOL ? *DROPTOL : 0.0;
    mem = MEM ? *MEM : 0.0;
    gap = *GAP;
  }
  // everything the double driver may have written, rounded into the caller's arrays
  void store(S* A, S* B, float* EIGS, float* RES, S* X, float* SHIFT, float* DROPTOL, float* MEM, float* GAP) {
    if (A && !diag_only) narrow(a.data(), A, nnz_a);
    if (B && !diag_only) narrow(b.data(), B, nnz_b);
    narrow(x.data(), X, (long)x.size());
    narrow(eigs.data(), EIGS, (long)eigs.size());
    narrow(res.data(), RES, (long)res.size());
    if (SHIFT) *SHIFT = (float)shift;
    if (DROPTOL) *DROPTOL = (float)droptol;
    if (MEM) *MEM = (float)mem;
    *GAP = (float)gap;
  }
  // the request's input vector into the caller's X, its results back
  void hand_out(S* X) {
    if (ijob == 2) narrow(x.data() + (ndx2 - 1), X + (ndx2 - 1), n);
    else narrow(x.data() + (ndx1 - 1), X + (ndx1 - 1), n);
  }
  void take_back(const S* X, bool gep) {
    if (ijob == 2) {
      widen(X + (ndx1 - 1), x.data() + (ndx1 - 1), n);
      return;
    }
    if (ijob == 1 || ijob == 3) widen(X + (ndx2 - 1), x.data() + (ndx2 - 1), n);
    if (gep && (ijob == 1 || ijob == 4)) widen(X + (ndx3 - 1), x.data() + (ndx3 - 1), n);
  }
};

// Host exceptions (allocation of the widened copies) must not cross the C
// ABI: they end the call with INFO = -54330, the library's code for a failure
// outside the algorithm.
template <class F> void guarded(int* INFO, F&& body) {
  try {
    body();
  } catch (...) {
    if (INFO) *INFO = -54330;
  }
}

template <class S> Copies<S>& revcom_copies(int which) {
  static Copies<S> c[2];  // 0: PJDREVCOM forms, 1: JDREVCOM forms
  return c[which];
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- SPJD ----
JDG_SAPI void JDG_S(spjd_)(int* N, float* A, int* JA, int* IA, float* EIGS, float* RES, float* X, int* LX, int* NEIG,
                   float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT,
                   float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<float> c;
    c.load(*N, A, JA, IA, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    JDG_S(dpjd_)(N, c.a.data(), JA, IA, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE,
          ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IPRINT, INFO, &c.gap);
    c.store(A, nullptr, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
  });
}

JDG_SAPI void JDG_S(spjd_gep_)(int* N, float* A, int* JA, int* IA, float* B, int* JB, int* IB, float* EIGS, float* RES,
                       float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER,
                       float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO,
                       float* GAP) {
  guarded(INFO, [&] {
    Copies<float> c;
    c.load(*N, A, JA, IA, B, IB, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    JDG_S(dpjd_gep_)(N, c.a.data(), JA, IA, c.b.data(), JB, IB, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma,
              ISEARCH, NINIT, MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IPRINT, INFO, &c.gap);
    c.store(A, B, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
  });
}

JDG_SAPI void JDG_S(spjdrevcom_)(int* N, float* A, int* JA, int* IA, float* EIGS, float* RES, float* X, int* LX, int* NEIG,
                         float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT,
                         float* DROPTOL, float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                         int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<float>& c = revcom_copies<float>(0);
    if (*IJOB == 0) c.load(*N, A, JA, IA, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    else c.take_back(X, false);
    JDG_S(dpjdrevcom_)(N, c.a.data(), JA, IA, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT,
                MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IJOB, NDX1, NDX2, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(A, nullptr, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(spjdrevcom_gep_)(int* N, float* A, int* JA, int* IA, float* B, int* JB, int* IB, float* EIGS, float* RES,
                             float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE,
                             int* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IJOB,
                             int* NDX1, int* NDX2, int* NDX3, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<float>& c = revcom_copies<float>(0);
    if (*IJOB == 0) c.load(*N, A, JA, IA, B, IB, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    else c.take_back(X, true);
    JDG_S(dpjdrevcom_gep_)(N, c.a.data(), JA, IA, c.b.data(), JB, IB, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG,
                    &c.sigma, ISEARCH, NINIT, MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IJOB, NDX1,
                    NDX2, NDX3, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(A, B, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.ndx3 = *NDX3;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(sjdrevcom_)(int* N, float* EIGS, float* RES, float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                        int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                        int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<float>& c = revcom_copies<float>(1);
    if (*IJOB == 0)
      c.load(*N, nullptr, nullptr, nullptr, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, nullptr, nullptr, nullptr, GAP);
    else c.take_back(X, false);
    JDG_S(djdrevcom_)(N, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE, ITER, &c.tol,
               IJOB, NDX1, NDX2, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(nullptr, nullptr, EIGS, RES, X, nullptr, nullptr, nullptr, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(sjdrevcom_gep_)(int* N, float* EIGS, float* RES, float* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                            int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1, int* NDX2,
                            int* NDX3, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<float>& c = revcom_copies<float>(1);
    if (*IJOB == 0)
      c.load(*N, nullptr, nullptr, nullptr, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, nullptr, nullptr, nullptr, GAP);
    else c.take_back(X, true);
    JDG_S(djdrevcom_gep_)(N, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE, ITER,
                   &c.tol, IJOB, NDX1, NDX2, NDX3, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(nullptr, nullptr, EIGS, RES, X, nullptr, nullptr, nullptr, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.ndx3 = *NDX3;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(spjdcleanup_)(void) {
  revcom_copies<float>(0) = Copies<float>();
  revcom_copies<float>(1) = Copies<float>();
  JDG_S(dpjdcleanup_)();
}

// ---------------------------------------------------------------- CPJD ----
JDG_SAPI void JDG_S(cpjd_)(int* N, jdg_ccomplex* A, int* JA, int* IA, float* EIGS, float* RES, jdg_ccomplex* X, int* LX,
                   int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL,
                   float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf> c;
    c.load(*N, A, JA, IA, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    JDG_S(zpjd_)(N, c.a.data(), JA, IA, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE,
          ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IPRINT, INFO, &c.gap);
    c.store(A, nullptr, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
  });
}

JDG_SAPI void JDG_S(cpjd_gep_)(int* N, jdg_ccomplex* A, int* JA, int* IA, jdg_ccomplex* B, int* JB, int* IB, float* EIGS,
                       float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT,
                       int* MADSPACE, int* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL,
                       int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf> c;
    c.load(*N, A, JA, IA, B, IB, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    JDG_S(zpjd_gep_)(N, c.a.data(), JA, IA, c.b.data(), JB, IB, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma,
              ISEARCH, NINIT, MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IPRINT, INFO, &c.gap);
    c.store(A, B, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
  });
}

JDG_SAPI void JDG_S(cpjdrevcom_)(int* N, jdg_ccomplex* A, int* JA, int* IA, float* EIGS, float* RES, jdg_ccomplex* X, int* LX,
                         int* NEIG, float* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL,
                         float* SHIFT, float* DROPTOL, float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2,
                         int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf>& c = revcom_copies<cf>(0);
    if (*IJOB == 0) c.load(*N, A, JA, IA, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    else c.take_back(X, false);
    JDG_S(zpjdrevcom_)(N, c.a.data(), JA, IA, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT,
                MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IJOB, NDX1, NDX2, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(A, nullptr, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(cpjdrevcom_gep_)(int* N, jdg_ccomplex* A, int* JA, int* IA, jdg_ccomplex* B, int* JB, int* IB,
                             float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA, int* ISEARCH,
                             int* NINIT, int* MADSPACE, int* ITER, float* TOL, float* SHIFT, float* DROPTOL,
                             float* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3, int* IPRINT,
                             int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf>& c = revcom_copies<cf>(0);
    if (*IJOB == 0) c.load(*N, A, JA, IA, B, IB, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, SHIFT, DROPTOL, MEM, GAP);
    else c.take_back(X, true);
    JDG_S(zpjdrevcom_gep_)(N, c.a.data(), JA, IA, c.b.data(), JB, IB, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG,
                    &c.sigma, ISEARCH, NINIT, MADSPACE, ITER, &c.tol, &c.shift, &c.droptol, &c.mem, ICNTL, IJOB, NDX1,
                    NDX2, NDX3, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(A, B, EIGS, RES, X, SHIFT, DROPTOL, MEM, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.ndx3 = *NDX3;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(cjdrevcom_)(int* N, float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA,
                        int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1,
                        int* NDX2, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf>& c = revcom_copies<cf>(1);
    if (*IJOB == 0)
      c.load(*N, nullptr, nullptr, nullptr, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, nullptr, nullptr, nullptr, GAP);
    else c.take_back(X, false);
    JDG_S(zjdrevcom_)(N, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE, ITER, &c.tol,
               IJOB, NDX1, NDX2, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(nullptr, nullptr, EIGS, RES, X, nullptr, nullptr, nullptr, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(cjdrevcom_gep_)(int* N, float* EIGS, float* RES, jdg_ccomplex* X, int* LX, int* NEIG, float* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, float* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, float* GAP) {
  guarded(INFO, [&] {
    Copies<cf>& c = revcom_copies<cf>(1);
    if (*IJOB == 0)
      c.load(*N, nullptr, nullptr, nullptr, nullptr, nullptr, EIGS, RES, X, *LX, *NEIG, SIGMA, TOL, nullptr, nullptr, nullptr, GAP);
    else c.take_back(X, true);
    JDG_S(zjdrevcom_gep_)(N, c.eigs.data(), c.res.data(), c.x.data(), LX, NEIG, &c.sigma, ISEARCH, NINIT, MADSPACE, ITER,
                   &c.tol, IJOB, NDX1, NDX2, NDX3, IPRINT, INFO, &c.gap);
    c.ijob = *IJOB;
    if (*IJOB == 0) {
      c.store(nullptr, nullptr, EIGS, RES, X, nullptr, nullptr, nullptr, GAP);
      return;
    }
    c.ndx1 = *NDX1;
    c.ndx2 = *NDX2;
    c.ndx3 = *NDX3;
    c.hand_out(X);
  });
}

JDG_SAPI void JDG_S(cpjdcleanup_)(void) {
  revcom_copies<cf>(0) = Copies<cf>();
  revcom_copies<cf>(1) = Copies<cf>();
  JDG_S(zpjdcleanup_)();
}

}  // extern "C"
