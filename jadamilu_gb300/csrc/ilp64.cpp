// 64-bit-integer drivers (include/jadamilu_gb300_ilp64.h) in front of the
// 32-bit ones of driver.cu, which this library compiles under the jdg_i32_
// prefix (JDG_ILP64_INNER).  Every call narrows the integer scalars and the
// CSR index arrays to 32 bits, calls the 32-bit driver and widens what it
// wrote back (NEIG, ITER, INFO, ICNTL, IJOB, NDX*, and the row entries of JA,
// which the drivers reorder so that the diagonal comes first).  The 32-bit
// copies live in one static state per driver: a reverse-communication solve
// keeps using them between calls, so they are loaded only when IJOB = 0.
// Values that do not fit in 32 bits return INFO = -1.
#include <climits>
#include <cstdint>
#include <vector>

#include "../../include/jadamilu_gb300_ilp64.h"

using I8 = jdg_i8;
using Z = jdg64_zcomplex;
using CF = jdg64_ccomplex;

extern "C" {
void jdg_i32_dpjd_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*,
                     double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_dpjd_gep_(int*, double*, int*, int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*,
                         int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_dpjdrevcom_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*,
                           double*, double*, double*, double*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_dpjdrevcom_gep_(int*, double*, int*, int*, double*, int*, int*, double*, double*, double*, int*, int*, double*,
                               int*, int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, int*,
                               int*, int*, int*, double*);
void jdg_i32_djdrevcom_(int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*, double*, int*, int*,
                          int*, int*, int*, double*);
void jdg_i32_djdrevcom_gep_(int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*, double*, int*,
                              int*, int*, int*, int*, int*, double*);
void jdg_i32_dpjdcleanup_(void);
void jdg_i32_zpjd_(int*, Z*, int*, int*, double*, double*, Z*, int*, int*, double*, int*, int*, int*, int*,
                     double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_zpjd_gep_(int*, Z*, int*, int*, Z*, int*, int*, double*, double*, Z*, int*, int*, double*, int*,
                         int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_zpjdrevcom_(int*, Z*, int*, int*, double*, double*, Z*, int*, int*, double*, int*, int*, int*, int*,
                           double*, double*, double*, double*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_zpjdrevcom_gep_(int*, Z*, int*, int*, Z*, int*, int*, double*, double*, Z*, int*, int*, double*,
                               int*, int*, int*, int*, double*, double*, double*, double*, int*, int*, int*, int*,
                               int*, int*, int*, double*);
void jdg_i32_zjdrevcom_(int*, double*, double*, Z*, int*, int*, double*, int*, int*, int*, int*, double*, int*, int*,
                          int*, int*, int*, double*);
void jdg_i32_zjdrevcom_gep_(int*, double*, double*, Z*, int*, int*, double*, int*, int*, int*, int*, double*, int*,
                              int*, int*, int*, int*, int*, double*);
void jdg_i32_zpjdcleanup_(void);
void jdg_i32_spjd_(int*, float*, int*, int*, float*, float*, float*, int*, int*, float*, int*, int*, int*, int*,
                     float*, float*, float*, float*, int*, int*, int*, float*);
void jdg_i32_spjd_gep_(int*, float*, int*, int*, float*, int*, int*, float*, float*, float*, int*, int*, float*, int*,
                         int*, int*, int*, float*, float*, float*, float*, int*, int*, int*, float*);
void jdg_i32_spjdrevcom_(int*, float*, int*, int*, float*, float*, float*, int*, int*, float*, int*, int*, int*, int*,
                           float*, float*, float*, float*, int*, int*, int*, int*, int*, int*, float*);
void jdg_i32_spjdrevcom_gep_(int*, float*, int*, int*, float*, int*, int*, float*, float*, float*, int*, int*, float*,
                               int*, int*, int*, int*, float*, float*, float*, float*, int*, int*, int*, int*,
                               int*, int*, int*, float*);
void jdg_i32_sjdrevcom_(int*, float*, float*, float*, int*, int*, float*, int*, int*, int*, int*, float*, int*, int*,
                          int*, int*, int*, float*);
void jdg_i32_sjdrevcom_gep_(int*, float*, float*, float*, int*, int*, float*, int*, int*, int*, int*, float*, int*,
                              int*, int*, int*, int*, int*, float*);
void jdg_i32_spjdcleanup_(void);
void jdg_i32_cpjd_(int*, CF*, int*, int*, float*, float*, CF*, int*, int*, float*, int*, int*, int*, int*,
                     float*, float*, float*, float*, int*, int*, int*, float*);
void jdg_i32_cpjd_gep_(int*, CF*, int*, int*, CF*, int*, int*, float*, float*, CF*, int*, int*, float*, int*,
                         int*, int*, int*, float*, float*, float*, float*, int*, int*, int*, float*);
void jdg_i32_cpjdrevcom_(int*, CF*, int*, int*, float*, float*, CF*, int*, int*, float*, int*, int*, int*, int*,
                           float*, float*, float*, float*, int*, int*, int*, int*, int*, int*, float*);
void jdg_i32_cpjdrevcom_gep_(int*, CF*, int*, int*, CF*, int*, int*, float*, float*, CF*, int*, int*, float*,
                               int*, int*, int*, int*, float*, float*, float*, float*, int*, int*, int*, int*,
                               int*, int*, int*, float*);
void jdg_i32_cjdrevcom_(int*, float*, float*, CF*, int*, int*, float*, int*, int*, int*, int*, float*, int*, int*,
                          int*, int*, int*, float*);
void jdg_i32_cjdrevcom_gep_(int*, float*, float*, CF*, int*, int*, float*, int*, int*, int*, int*, float*, int*,
                              int*, int*, int*, int*, int*, float*);
void jdg_i32_cpjdcleanup_(void);
void jdg_i32_pjd_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*,
                  double*, double*, double*, double*, int*, int*, int*, double*);
void jdg_i32_pjdrevcom_(int*, double*, int*, int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*,
                        double*, double*, double*, double*, int*, int*, int*, int*, int*, int*, double*);
void jdg_i32_jdrevcom_(int*, double*, double*, double*, int*, int*, double*, int*, int*, int*, int*, double*, int*, int*,
                       int*, int*, int*, double*);
void jdg_i32_pjdcleanup_(void);
}

namespace {

bool fits(I8 v) { return v >= INT_MIN && v <= INT_MAX; }

// 32-bit copy of a one-triangle CSR (IA: n+1 row starts, JA: column of each
// entry, 1-based).  With JA(1) < 0 (diagonal preconditioning) the drivers
// read JA(1) only.
struct Idx {
  std::vector<int> ia, ja;
  bool diag_only = false;
  bool load(I8 n, const I8* IA, const I8* JA) {
    diag_only = JA[0] < 0;
    if (diag_only) {
      ja.assign(1, (int)(fits(JA[0]) ? JA[0] : -1));
      ia.assign(1, (int)(fits(IA[0]) ? IA[0] : 1));
      return true;
    }
    ia.resize((size_t)n + 1);
    for (I8 i = 0; i <= n; ++i) {
      if (!fits(IA[i])) return false;
      ia[(size_t)i] = (int)IA[i];
    }
    const I8 nnz = IA[n] - 1;
    if (nnz < 0 || !fits(nnz)) return false;
    ja.resize((size_t)nnz);
    for (I8 q = 0; q < nnz; ++q) {
      if (!fits(JA[q])) return false;
      ja[(size_t)q] = (int)JA[q];
    }
    return true;
  }
  void store_ja(I8* JA) const {
    if (diag_only) return;
    for (size_t q = 0; q < ja.size(); ++q) JA[q] = ja[q];
  }
};

struct State {
  int n = 0, lx = 0, neig = 0, isearch = 0, ninit = 0, madspace = 0, iter = 0, iprint = 0, info = 0;
  int icntl[5] = {0, 0, 0, 0, 0};
  int ijob = 0, ndx1 = 0, ndx2 = 0, ndx3 = 0;
  Idx a, b;
  bool load(I8* N, I8* LX, I8* NEIG, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, I8* ICNTL, I8* IPRINT) {
    const I8 v[] = {*N, *LX, *NEIG, *ISEARCH, *NINIT, *MADSPACE, *ITER, *IPRINT};
    for (I8 x : v)
      if (!fits(x)) return false;
    if (*N < 1) return false;
    n = (int)*N;
    lx = (int)*LX;
    neig = (int)*NEIG;
    isearch = (int)*ISEARCH;
    ninit = (int)*NINIT;
    madspace = (int)*MADSPACE;
    iter = (int)*ITER;
    iprint = (int)*IPRINT;
    if (ICNTL)
      for (int i = 0; i < 5; ++i) {
        if (!fits(ICNTL[i])) return false;
        icntl[i] = (int)ICNTL[i];
      }
    return true;
  }
  void store(I8* NEIG, I8* ITER, I8* ICNTL, I8* INFO) const {
    *NEIG = neig;
    *ITER = iter;
    *INFO = info;
    if (ICNTL)
      for (int i = 0; i < 5; ++i) ICNTL[i] = icntl[i];
  }
};

}  // namespace

extern "C" {
JDG64_API void dpjd_(I8* N, double* A, I8* JA, I8* IA, double* EIGS, double* RES, double* X, I8* LX, I8* NEIG,
                    double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, double* SHIFT,
                    double* DROPTOL, double* MEM, I8* ICNTL, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA)) {
    *INFO = -1;
    return;
  }
  jdg_i32_dpjd_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void dpjd_gep_(I8* N, double* A, I8* JA, I8* IA, double* B, I8* JB, I8* IB, double* EIGS, double* RES,
                        double* X, I8* LX, I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER,
                        double* TOL, double* SHIFT, double* DROPTOL, double* MEM, I8* ICNTL, I8* IPRINT, I8* INFO,
                        double* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA) ||
      !s.b.load(*N, IB, JB)) {
    *INFO = -1;
    return;
  }
  jdg_i32_dpjd_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X, &s.lx,
                     &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl,
                     &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.b.store_ja(JB);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void dpjdrevcom_(I8* N, double* A, I8* JA, I8* IA, double* EIGS, double* RES, double* X, I8* LX,
                          I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL,
                          double* SHIFT, double* DROPTOL, double* MEM, I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2,
                          I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 &&
      (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_dpjdrevcom_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.iprint, &s.info,
          GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) s.a.store_ja(JA);
}
JDG64_API void dpjdrevcom_gep_(I8* N, double* A, I8* JA, I8* IA, double* B, I8* JB, I8* IB, double* EIGS,
                              double* RES, double* X, I8* LX, I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT,
                              I8* MADSPACE, I8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                              I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) ||
                     !s.a.load(*N, IA, JA) || !s.b.load(*N, IB, JB))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_dpjdrevcom_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X,
                           &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL,
                           MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) {
    s.a.store_ja(JA);
    s.b.store_ja(JB);
  }
}
JDG64_API void djdrevcom_(I8* N, double* EIGS, double* RES, double* X, I8* LX, I8* NEIG, double* SIGMA,
                         I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, I8* IJOB, I8* NDX1, I8* NDX2,
                         I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_djdrevcom_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, &s.ijob,
          &s.ndx1, &s.ndx2, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void djdrevcom_gep_(I8* N, double* EIGS, double* RES, double* X, I8* LX, I8* NEIG, double* SIGMA,
                             I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, I8* IJOB, I8* NDX1,
                             I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_djdrevcom_gep_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter,
                          TOL, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void dpjdcleanup_(void) { jdg_i32_dpjdcleanup_(); }
JDG64_API void zpjd_(I8* N, Z* A, I8* JA, I8* IA, double* EIGS, double* RES, Z* X, I8* LX, I8* NEIG,
                    double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, double* SHIFT,
                    double* DROPTOL, double* MEM, I8* ICNTL, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA)) {
    *INFO = -1;
    return;
  }
  jdg_i32_zpjd_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void zpjd_gep_(I8* N, Z* A, I8* JA, I8* IA, Z* B, I8* JB, I8* IB, double* EIGS, double* RES,
                        Z* X, I8* LX, I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER,
                        double* TOL, double* SHIFT, double* DROPTOL, double* MEM, I8* ICNTL, I8* IPRINT, I8* INFO,
                        double* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA) ||
      !s.b.load(*N, IB, JB)) {
    *INFO = -1;
    return;
  }
  jdg_i32_zpjd_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X, &s.lx,
                     &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl,
                     &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.b.store_ja(JB);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void zpjdrevcom_(I8* N, Z* A, I8* JA, I8* IA, double* EIGS, double* RES, Z* X, I8* LX,
                          I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL,
                          double* SHIFT, double* DROPTOL, double* MEM, I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2,
                          I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 &&
      (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_zpjdrevcom_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.iprint, &s.info,
          GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) s.a.store_ja(JA);
}
JDG64_API void zpjdrevcom_gep_(I8* N, Z* A, I8* JA, I8* IA, Z* B, I8* JB, I8* IB, double* EIGS,
                              double* RES, Z* X, I8* LX, I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT,
                              I8* MADSPACE, I8* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                              I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) ||
                     !s.a.load(*N, IA, JA) || !s.b.load(*N, IB, JB))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_zpjdrevcom_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X,
                           &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL,
                           MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) {
    s.a.store_ja(JA);
    s.b.store_ja(JB);
  }
}
JDG64_API void zjdrevcom_(I8* N, double* EIGS, double* RES, Z* X, I8* LX, I8* NEIG, double* SIGMA,
                         I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, I8* IJOB, I8* NDX1, I8* NDX2,
                         I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_zjdrevcom_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, &s.ijob,
          &s.ndx1, &s.ndx2, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void zjdrevcom_gep_(I8* N, double* EIGS, double* RES, Z* X, I8* LX, I8* NEIG, double* SIGMA,
                             I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, I8* IJOB, I8* NDX1,
                             I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_zjdrevcom_gep_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter,
                          TOL, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void zpjdcleanup_(void) { jdg_i32_zpjdcleanup_(); }
// single-precision drivers: the same narrowing around the inner REAL / COMPLEX drivers
JDG64_API void spjd_(I8* N, float* A, I8* JA, I8* IA, float* EIGS, float* RES, float* X, I8* LX, I8* NEIG,
                    float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, float* SHIFT,
                    float* DROPTOL, float* MEM, I8* ICNTL, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA)) {
    *INFO = -1;
    return;
  }
  jdg_i32_spjd_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void spjd_gep_(I8* N, float* A, I8* JA, I8* IA, float* B, I8* JB, I8* IB, float* EIGS, float* RES,
                        float* X, I8* LX, I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER,
                        float* TOL, float* SHIFT, float* DROPTOL, float* MEM, I8* ICNTL, I8* IPRINT, I8* INFO,
                        float* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA) ||
      !s.b.load(*N, IB, JB)) {
    *INFO = -1;
    return;
  }
  jdg_i32_spjd_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X, &s.lx,
                     &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl,
                     &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.b.store_ja(JB);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void spjdrevcom_(I8* N, float* A, I8* JA, I8* IA, float* EIGS, float* RES, float* X, I8* LX,
                          I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL,
                          float* SHIFT, float* DROPTOL, float* MEM, I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2,
                          I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 &&
      (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_spjdrevcom_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.iprint, &s.info,
          GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) s.a.store_ja(JA);
}
JDG64_API void spjdrevcom_gep_(I8* N, float* A, I8* JA, I8* IA, float* B, I8* JB, I8* IB, float* EIGS,
                              float* RES, float* X, I8* LX, I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT,
                              I8* MADSPACE, I8* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM,
                              I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) ||
                     !s.a.load(*N, IA, JA) || !s.b.load(*N, IB, JB))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_spjdrevcom_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X,
                           &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL,
                           MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) {
    s.a.store_ja(JA);
    s.b.store_ja(JB);
  }
}
JDG64_API void sjdrevcom_(I8* N, float* EIGS, float* RES, float* X, I8* LX, I8* NEIG, float* SIGMA,
                         I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, I8* IJOB, I8* NDX1, I8* NDX2,
                         I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_sjdrevcom_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, &s.ijob,
          &s.ndx1, &s.ndx2, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void sjdrevcom_gep_(I8* N, float* EIGS, float* RES, float* X, I8* LX, I8* NEIG, float* SIGMA,
                             I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, I8* IJOB, I8* NDX1,
                             I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_sjdrevcom_gep_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter,
                          TOL, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void spjdcleanup_(void) { jdg_i32_spjdcleanup_(); }
JDG64_API void cpjd_(I8* N, CF* A, I8* JA, I8* IA, float* EIGS, float* RES, CF* X, I8* LX, I8* NEIG,
                    float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, float* SHIFT,
                    float* DROPTOL, float* MEM, I8* ICNTL, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA)) {
    *INFO = -1;
    return;
  }
  jdg_i32_cpjd_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void cpjd_gep_(I8* N, CF* A, I8* JA, I8* IA, CF* B, I8* JB, I8* IB, float* EIGS, float* RES,
                        CF* X, I8* LX, I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER,
                        float* TOL, float* SHIFT, float* DROPTOL, float* MEM, I8* ICNTL, I8* IPRINT, I8* INFO,
                        float* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA) ||
      !s.b.load(*N, IB, JB)) {
    *INFO = -1;
    return;
  }
  jdg_i32_cpjd_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X, &s.lx,
                     &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl,
                     &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.b.store_ja(JB);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void cpjdrevcom_(I8* N, CF* A, I8* JA, I8* IA, float* EIGS, float* RES, CF* X, I8* LX,
                          I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL,
                          float* SHIFT, float* DROPTOL, float* MEM, I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2,
                          I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 &&
      (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_cpjdrevcom_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.iprint, &s.info,
          GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) s.a.store_ja(JA);
}
JDG64_API void cpjdrevcom_gep_(I8* N, CF* A, I8* JA, I8* IA, CF* B, I8* JB, I8* IB, float* EIGS,
                              float* RES, CF* X, I8* LX, I8* NEIG, float* SIGMA, I8* ISEARCH, I8* NINIT,
                              I8* MADSPACE, I8* ITER, float* TOL, float* SHIFT, float* DROPTOL, float* MEM,
                              I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) ||
                     !s.a.load(*N, IA, JA) || !s.b.load(*N, IB, JB))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_cpjdrevcom_gep_(&s.n, A, s.a.ja.data(), s.a.ia.data(), B, s.b.ja.data(), s.b.ia.data(), EIGS, RES, X,
                           &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, SHIFT, DROPTOL,
                           MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) {
    s.a.store_ja(JA);
    s.b.store_ja(JB);
  }
}
JDG64_API void cjdrevcom_(I8* N, float* EIGS, float* RES, CF* X, I8* LX, I8* NEIG, float* SIGMA,
                         I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, I8* IJOB, I8* NDX1, I8* NDX2,
                         I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_cjdrevcom_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, &s.ijob,
          &s.ndx1, &s.ndx2, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void cjdrevcom_gep_(I8* N, float* EIGS, float* RES, CF* X, I8* LX, I8* NEIG, float* SIGMA,
                             I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, float* TOL, I8* IJOB, I8* NDX1,
                             I8* NDX2, I8* NDX3, I8* IPRINT, I8* INFO, float* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_cjdrevcom_gep_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter,
                          TOL, &s.ijob, &s.ndx1, &s.ndx2, &s.ndx3, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  *NDX3 = s.ndx3;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void cpjdcleanup_(void) { jdg_i32_cpjdcleanup_(); }
JDG64_API void pjd_(I8* N, double* A, I8* JA, I8* IA, double* EIGS, double* RES, double* X, I8* LX, I8* NEIG,
                    double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, double* SHIFT,
                    double* DROPTOL, double* MEM, I8* ICNTL, I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA)) {
    *INFO = -1;
    return;
  }
  jdg_i32_pjd_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.iprint, &s.info, GAP);
  s.a.store_ja(JA);
  s.store(NEIG, ITER, ICNTL, INFO);
}
JDG64_API void pjdrevcom_(I8* N, double* A, I8* JA, I8* IA, double* EIGS, double* RES, double* X, I8* LX,
                          I8* NEIG, double* SIGMA, I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL,
                          double* SHIFT, double* DROPTOL, double* MEM, I8* ICNTL, I8* IJOB, I8* NDX1, I8* NDX2,
                          I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 &&
      (!s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, ICNTL, IPRINT) || !s.a.load(*N, IA, JA))) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_pjdrevcom_(&s.n, A, s.a.ja.data(), s.a.ia.data(), EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit,
          &s.madspace, &s.iter, TOL, SHIFT, DROPTOL, MEM, s.icntl, &s.ijob, &s.ndx1, &s.ndx2, &s.iprint, &s.info,
          GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, ICNTL, INFO);
  if (s.ijob == 0) s.a.store_ja(JA);
}
JDG64_API void jdrevcom_(I8* N, double* EIGS, double* RES, double* X, I8* LX, I8* NEIG, double* SIGMA,
                         I8* ISEARCH, I8* NINIT, I8* MADSPACE, I8* ITER, double* TOL, I8* IJOB, I8* NDX1, I8* NDX2,
                         I8* IPRINT, I8* INFO, double* GAP) {
  static State s;
  if (*IJOB == 0 && !s.load(N, LX, NEIG, ISEARCH, NINIT, MADSPACE, ITER, nullptr, IPRINT)) {
    *INFO = -1;
    return;
  }
  s.ijob = (int)*IJOB;
  jdg_i32_jdrevcom_(&s.n, EIGS, RES, X, &s.lx, &s.neig, SIGMA, &s.isearch, &s.ninit, &s.madspace, &s.iter, TOL, &s.ijob,
          &s.ndx1, &s.ndx2, &s.iprint, &s.info, GAP);
  *IJOB = s.ijob;
  *NDX1 = s.ndx1;
  *NDX2 = s.ndx2;
  s.store(NEIG, ITER, nullptr, INFO);
}
JDG64_API void pjdcleanup_(void) { jdg_i32_pjdcleanup_(); }

}  // extern "C"
