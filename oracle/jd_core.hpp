// Test infrastructure only: CPU restatement of the Jacobi-Davidson core of
// JADAMILU, used as the oracle that the GPU library is checked against.
//
// Follows src/jd/JDaux.F of the reference:
//   JDRVCOM   :1391-2415  (outer loop, locking, restart, expansion, final RR)
//   LSOLREVCOM:2989-3268  (inner CG / smoothed-CG "sQMR")
//   STOPTEST  :2542-2672  (inner stopping rule)
//   REPGS     :2674-2753  (DGKS / classical Gram-Schmidt)
//   SOLPROJEP :3271-3358  (projected J x J eigenproblem)
//   SHRINK    :2418-2462  (restart by QR of the kept Ritz coefficients)
//   SORTEV    :2464-2540  (ordering of eigenpairs)
// The workspace X keeps the reference layout (JDaux.F:1534-1567) because the
// reverse-communication offsets and the eigenvector output are defined on it.
// Instead of returning to the caller (IJOB=1..4) the oracle calls back.
// Nothing here is linked into the GPU library.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../jadamilu_gb300/csrc/small_dense.hpp"

namespace orc {
using namespace jdd;

// Values that JDRVCOM shares with the preconditioner-aware driver through
// the COMMON block /JDRVCOMJD/ (JDaux.F:47-48).
struct JdShared {
  double timeilu = 0, rinit = 0, rcurr = 0, rcum = 0, shift1 = 0;
  bool flagcg = false;
};

template <class T> struct JdCallbacks {
  // which = 1: y = A x and (GEP) by = B x;  3: y = A x;  4: by = B x
  void (*matvec)(void* ctx, int which, const T* x, T* y, T* by);
  // sol = Prec^{-1} rhs  (JDRVCOM's IJOB=2: Prec X(NDX1) = X(NDX2))
  void (*precond)(void* ctx, const T* rhs, T* sol);
  void* ctx;
};

struct StopState {
  int istag = 0, istt = 0;
  bool posdef = false, toupdate = false;
  double g0 = 0, gs = 0, gtrs = 0, gkmin = 0, bk = 0, beta = 0, tn = 0, un2 = -1, gkm1 = 0, alp = 1;
};

// 48-bit linear congruential uniform(0,1) stream for the random restart of
// REPGS (the reference uses LAPACK's DLARNV with seed 1,7,11,17).
struct Lcg48 {
  unsigned long long s = 0x1234ABCD330EULL;
  double next() {
    s = (s * 0x5DEECE66DULL + 0xB) & ((1ULL << 48) - 1);
    return ((double)(s >> 5) + 0.5) / (double)(1ULL << 43);
  }
};

template <class T> struct JdCore {
  JdShared* sh;
  JdCallbacks<T> cb;
  StopState st;
  Lcg48 rng;
  double alpha_cg = 0;  // SAVE'd ALPHA of the inner solver
  int istag = 0;        // SAVE'd ISTAG of JDRVCOM

  // REPGS: orthogonalise w against the JV columns of V (B-inner product via BV).
  void repgs(long N, const T* V, long ldv, const T* BV, long ldbv, long JV, T* w, T* y, double epsm, int gam) {
    bool nrnd = true;
    if (JV <= 0) return;
    if (gam < 0) {
      gemv_c(N, JV, T(1), BV, ldbv, w, T(0), y);
      gemv_n(N, JV, T(-1), V, ldv, y, T(1), w);
      return;
    }
    for (;;) {
      double nrn = nrm2(N, w), nr = epsm * nrn, nro;
      if (nrnd) fillv(JV, T(0), y);
      bool small = false;
      do {
        nro = nrn;
        gemv_c(N, JV, T(1), BV, ldbv, w, T(0), y + JV);
        gemv_n(N, JV, T(-1), V, ldv, y + JV, T(1), w);
        nrn = nrm2(N, w);
        if (nrnd) axpy(JV, T(1), y + JV, y);
        if (nrn <= nr) { small = true; break; }
      } while (nrn < 0.5 * nro);
      if (!small) { y[JV] = T(nrn); return; }
      if (gam == 1) {
        if (JV < N) {
          for (long i = 0; i < N; ++i) w[i] = T(rng.next());
          nrnd = false;
          continue;
        }
      } else {
        fillv(N, T(0), w);
        y[JV] = T(0);
      }
      return;
    }
  }

  // SORTEV: reorder eigenpairs.  it = +-2: by decreasing |eigs-sigma| (-2 then
  // rotates the last to the front); +-4: increasing eigs (also RES, and V2
  // when -4); otherwise decreasing eigs.
  void sortev(long N, long J, T* V, long ldv, T* V2, long ldv2, double* eigs, double* r, int it, double sigma) {
    if (J <= 1) return;
    std::vector<double> key(J);
    for (long i = 0; i < J; ++i) {
      if (it == 2 || it == -2) key[i] = -std::fabs(eigs[i] - sigma);
      else if (it == 4 || it == -4) key[i] = eigs[i];
      else key[i] = -eigs[i];
    }
    std::vector<long> iw(J);
    sort_index(J, key.data(), iw.data());
    if (it == -2) {
      long last = iw[J - 1];
      for (long i = J - 1; i > 0; --i) iw[i] = iw[i - 1];
      iw[0] = last;
    }
    std::vector<T> tv((size_t)N * J);
    for (long k = 0; k < J; ++k) copyv(N, V + iw[k] * ldv, tv.data() + k * N);
    for (long k = 0; k < J; ++k) copyv(N, tv.data() + k * N, V + k * ldv);
    if (it == -4) {
      for (long k = 0; k < J; ++k) copyv(N, V2 + iw[k] * ldv2, tv.data() + k * N);
      for (long k = 0; k < J; ++k) copyv(N, tv.data() + k * N, V2 + k * ldv2);
    }
    std::vector<double> te(J);
    for (long k = 0; k < J; ++k) te[k] = eigs[iw[k]];
    for (long k = 0; k < J; ++k) eigs[k] = te[k];
    if (it == 4 || it == -4) {
      for (long k = 0; k < J; ++k) te[k] = r[iw[k]];
      for (long k = 0; k < J; ++k) r[k] = te[k];
    }
  }

  // SOLPROJEP (JDaux.F:3271-3358): J x J projected eigenproblem.  |is|=2:
  // harmonic, sorted by decreasing |mu| -- generalized Hermitian MM y = mu NN y
  // for the standard problem; for the generalized problem MM is a general
  // matrix: NN^{-1} MM (Cholesky solve, POSV) and its right eigenvectors
  // (GEEV), real parts of the eigenvalues.  Otherwise standard on MM.  is = 3
  // writes all eigenvalues into NN's first column.
  void solprojep(long J, T* MM, T* NN, long ld, double& theta, double& theta2, double* w, int is, int& info, bool gep) {
    if (is == 2 || is == -2) {
      if (gep) {
        info = posv_u(J, NN, ld, MM, ld);
        if (info) return;
        copyv(ld * ld, MM, NN);
        info = geev_right(J, NN, ld, w, MM, ld);
        if (info) return;
        sortev(J, J, MM, ld, NN, ld, w, nullptr, is, 0.0);
        theta2 = w[1];
        return;
      }
      info = hegv(J, MM, ld, NN, ld, w);
      if (info) return;
      sortev(J, J, MM, ld, NN, ld, w, nullptr, is, 0.0);
      theta2 = w[1];
      return;
    }
    herm_full(J, MM, ld);
    info = heev(J, MM, ld, w);
    if (info) return;
    if (is == 3) {
      for (long i = 0; i < J; ++i) NN[i] = T(w[i]);
    } else {
      theta = w[0];
      theta2 = w[1];
    }
  }

  // SHRINK: keep span(V*U(:,1:J)) via the Q factor of U (K x J).
  void shrink(long N, long J, long K, const T* U, long ldu, T* V, T* W, T* BV, T* MM, T* NN, long ld, int iserch, bool gep) {
    std::vector<T> Q;
    householder_q(K, J, U, ldu, Q);
    right_mult(N, K, K, V, Q);
    right_mult(N, K, K, W, Q);
    if (gep) right_mult(N, K, K, BV, Q);
    auto congr = [&](T* M, bool herm) {
      if (herm)
        for (long i = 1; i < K; ++i)
          for (long j = 0; j < i; ++j) M[i + j * ld] = cj(M[j + i * ld]);
      std::vector<T> tmp(K * K), out(K * K);
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) {
          T s = T(0);
          for (long k = 0; k < K; ++k) s += M[i + k * ld] * Q[k + j * K];
          tmp[i + j * K] = s;
        }
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) {
          T s = T(0);
          for (long k = 0; k < K; ++k) s += cj(Q[k + i * K]) * tmp[k + j * K];
          out[i + j * K] = s;
        }
      for (long j = 0; j < K; ++j)
        for (long i = 0; i < K; ++i) M[i + j * ld] = out[i + j * K];
    };
    congr(MM, iserch != 2 || !gep);
    if (iserch == 2) congr(NN, true);
  }

  // STOPTEST (info in/out: -1/-2 first call, 0 continue, 1 stop)
  void stoptest(long N, const T* x, const T* bt, const T* bu, double tol, double& rk, double nbu, double& alprho,
                double& gk, T pcad, T pcr, double& theta, double eta, int& info, double trs, bool gep) {
    StopState& s = st;
    static thread_local T bkgep, bubt;
    if (info != 0) {
      s.posdef = (info == -1);
      s.istag = 0;
      s.istt = 0;
      s.g0 = rk;
      s.gkm1 = rk;
      s.gtrs = trs * s.g0;
      if (s.gtrs < tol) s.gtrs = tol;
      s.gs = s.gtrs;
      s.gkmin = s.g0;
      s.bk = theta - eta;
      if (gep) bkgep = T(theta - eta) + pcr;
      s.un2 = -1;
    }
    s.bk -= alprho;
    if (gep) {
      bkgep -= pcad;
      s.beta = ab(bkgep);
      gk = gk / nbu;
    } else {
      s.beta = std::fabs(s.bk);
    }
    if (gk < s.gkmin) { s.gkmin = gk; s.istag = 0; }
    if (gk > s.gkm1) { s.istag++; s.istt++; }
    bool stop = false;
    if (s.istag >= 25 || s.istt >= 100) stop = true;
    else if (s.gkmin >= s.gtrs) stop = false;
    else {
      s.toupdate = true;
      bool do13 = !(gk >= s.gs);
      for (;;) {
        if (do13) {
          if (gep) {
            s.tn = nrm2(N, bt) / nbu;
            bubt = -dotc(N, bu, bt) / (nbu * nbu);
            s.alp = ab(T(1) + bubt);
            s.tn = std::sqrt(re(cj(T(s.tn) + bubt) * (T(s.tn) - bubt))) / s.alp;
          } else {
            s.alp = 1;
            s.tn = nrm2(N, x);
          }
          s.un2 = 1 + s.tn * s.tn;
          s.toupdate = false;
          s.gs = (gk < 0.1 * s.g0) ? tol : 0.1 * s.g0;
          if (s.gs < tol) s.gs = tol;
        }
        if (gep) {
          if (s.beta < gk * s.tn) rk = std::sqrt((gk * gk + s.beta * s.beta) / s.un2) / s.alp;
          else rk = (gk + s.beta * s.tn) / (s.alp * s.un2);
        } else {
          rk = std::sqrt(gk * gk * s.un2 + s.tn * s.tn * s.beta * s.beta) / s.un2;
        }
        if (rk < tol && s.toupdate) { do13 = true; continue; }
        break;
      }
      double lim = 0.5 * tol * s.un2 * s.alp;
      if (rk < tol) stop = true;
      else if (gk * std::sqrt(s.un2) < 15 * s.tn * s.beta && s.beta * s.tn > lim) stop = true;
      else if (s.istag >= 3) stop = true;
      else if (s.istag >= 1 && s.beta * s.tn > lim && gk < s.gtrs) stop = true;
    }
    if (!stop) {
      info = 0;
      s.gkm1 = gk;
      return;
    }
    info = info > 1 ? info : 1;
    if (gep) alprho = s.un2 * s.alp * s.alp;
    theta = s.bk;
  }

  // The JD core.  Returns with INFO set like JDRVCOM; all matvecs and
  // preconditioner solves go through the callbacks.
  void run(long N, double* EIGS, double* RES, T* X, long LX, int& NEIG, double SIGMA, int ISEARCH, int NINIT,
           int MADSPACE, int& ITER, double TOL, int& INFO, double& GAP, bool GEP);
};

template <class T>
void JdCore<T>::run(long N, double* EIGS, double* RES, T* X, long LX, int& NEIG, double SIGMA, int ISEARCH,
                    int NINIT, int MADSPACE, int& ITER, double TOL, int& INFO, double& GAP, bool GEP) {
  const double EPSM = DBL_EPSILON * 0.5, RINF = DBL_MAX;
  JdShared& S = *sh;
  S.flagcg = true;
  bool neweig = true;
  S.rcum = 0;
  double RINITM = 1;
  INFO = 0;
  long MOD = MADSPACE;
  if (N < 2) INFO = -1;
  else if (NEIG <= 0) INFO = -5;
  else if (MADSPACE <= 2) INFO = -9;
  else if (N * (2 * MOD + NEIG + 4) + 3 * MOD * MOD + std::max(MOD * MOD, (long)NEIG) > LX) INFO = -10;
  else if (GEP && N * (3 * MOD + 2 * NEIG + 4) + 3 * MOD * MOD + std::max(MOD * MOD, (long)NEIG) > LX) INFO = -10;
  else if (ITER <= 0) INFO = -11;
  else if (TOL <= 0) INFO = -12;
  if (INFO != 0) return;
  MOD = std::min<long>(MADSPACE, N);
  const long NWANT = std::min<long>(NEIG, N);
  const int MVMAX = ITER;
  int ISERCH = std::min(ISEARCH, 2);  // JDaux.F:1531-1532 (the clamp at 0 is overwritten)
  // workspace (0-based offsets into X)
  const long XX = 0, VV = XX + NWANT * N, WW = VV + MOD * N;
  long BX, BV, MM;
  if (GEP) { BX = WW + MOD * N; BV = BX + NWANT * N; MM = BV + MOD * N; }
  else { BX = XX; BV = VV; MM = WW + MOD * N; }
  const long NN = MM + MOD * MOD, MP = NN + MOD * MOD, NP = MP + MOD * MOD;
  const long WCG = NP + std::max(MOD * MOD, NWANT);
  const long XCG2 = WW + (MOD - 1) * N, BT = BV + (MOD - 1) * N, REIG = WCG, YY = MP, YY2 = MP + MOD;
  const long WL = REIG + N, WL2 = WL + MOD, WL3 = WL2 + MOD;
  long UU = XX + (NWANT - 1) * N, BU = BX + (NWANT - 1) * N, KXP = VV, KBXP = BV;
  double* Wr = reinterpret_cast<double*>(X + REIG);  // SOLPROJEP's real W aliases X(REIG)
  const double EPSMSR = std::sqrt(EPSM);
  NEIG = 0;
  ITER = 0;
  double ETA1 = RINF, ETA0 = SIGMA, DELTA1 = RINF, NREIG = RINF, RESID = RINF, RNDIND = 0, DELTAO = 0;
  if (ISERCH == 0) ETA0 = RINF;
  const long MIDSPACE = (MOD + 1) / 2;
  bool INITFLG = false, UKNOWN = false, CONV = false;
  double THETA = 0, THETA2 = 0, THMT = 0, NBU = 1, NREIGP = 0, TRS = 0, ETA = 0, SCLR1 = 0, SCLR2 = 0, ALPRHO = 0,
         GK = 0;
  T AXPYALPHA = T(0), AXPYBETA = T(0);
  long J = 0, K = 0, IJ = 0;
  int IFO = 0;
  if (NINIT > MIDSPACE) {
    for (int ii = 1; ii < NINIT; ++ii)
      if (EIGS[ii] != EIGS[0]) INITFLG = true;
    if (INITFLG) {
      sortev(N, NINIT, X + XX, N, nullptr, N, EIGS, RES, ISERCH, SIGMA);
    } else {
      for (int ii = 0; ii < NINIT / 2; ++ii) {
        int jj = NINIT - 1 - ii;
        copyv(N, X + (long)jj * N, X + VV);
        copyv(N, X + (long)ii * N, X + (long)jj * N);
        copyv(N, X + VV, X + (long)ii * N);
      }
    }
  }
  INITFLG = false;

  auto bmatvec = [&](long x, long bx) { cb.matvec(cb.ctx, 4, X + x, nullptr, X + bx); };
  auto bnormalize = [&](long u, long bu, double& s) -> bool {  // B-normalise u (labels 15/45)
    s = re(dotc(N, X + u, X + bu));
    if (s <= 0) return false;
    s = std::sqrt(s);
    rscal(N, 1 / s, X + bu);
    return true;
  };

start_space:  // label 2
  if (NINIT <= NEIG) {
    J = 1;
    fillv(N, T(1), X + VV);
  } else {
    J = std::min<long>(NINIT - NEIG, MIDSPACE);
    IJ = NINIT - NEIG - J;
    if (IJ > 0) INITFLG = true;
    copyv(N * J, X + N * IJ, X + VV);
  }
  for (IJ = 1; IJ <= J; ++IJ) {  // labels 4-5
    long vj = VV + (IJ - 1) * N;
    repgs(N, X + KXP, N, X + KBXP, N, NEIG + IJ - 1, X + vj, X + WL, EPSM, 1);
    if (!GEP) {
      SCLR1 = (NEIG + IJ - 1 > 0) ? re(X[WL + NEIG + IJ - 1]) : nrm2(N, X + VV);
      rscal(N, 1 / SCLR1, X + vj);
    }
    cb.matvec(cb.ctx, 1, X + vj, X + WW + (IJ - 1) * N, X + BV + (IJ - 1) * N);
    ITER++;
    if (GEP) {
      long bvj = BV + (IJ - 1) * N;
      SCLR1 = re(dotc(N, X + vj, X + bvj));
      if (SCLR1 <= 0) goto err_bnotspd;
      SCLR1 = std::sqrt(SCLR1);
      rscal(N, 1 / SCLR1, X + bvj);
      rscal(N, 1 / SCLR1, X + vj);
      rscal(N, 1 / SCLR1, X + WW + (IJ - 1) * N);
    }
  }
  if (ISERCH == 2) {
    axpy(N * J, T(-SIGMA), X + BV, X + WW);
    for (long c = 0; c < J; ++c)  // NN = W^H W (upper)
      for (long r = 0; r <= c; ++r) X[NN + r + c * MOD] = dotc(N, X + WW + r * N, X + WW + c * N);
  }
  if (ISERCH == 2 && GEP) {
    for (long c = 0; c < J; ++c)
      for (long r = 0; r < J; ++r) X[MM + r + c * MOD] = dotc(N, X + WW + r * N, X + BV + c * N);
  } else {
    for (long c = 0; c < J; ++c)  // SYR2K: V^H W + W^H V, then halved
      for (long r = 0; r <= c; ++r)
        X[MM + r + c * MOD] = dotc(N, X + VV + r * N, X + WW + c * N) + dotc(N, X + WW + r * N, X + VV + c * N);
    rscal(MOD * MOD, 0.5, X + MM);
  }
  UKNOWN = (J <= 1);

main_loop:  // label 10: extraction
  copyv(MOD * MOD, X + MM, X + MP);
  if (ISERCH == 2) copyv(MOD * MOD, X + NN, X + NP);
  solprojep(J, X + MP, X + NP, MOD, THETA, THETA2, Wr, ISERCH, INFO, GEP);
  if (INFO != 0) goto err_lapack;
  if (!UKNOWN) {
    if (ISERCH == 2) {
      SCLR1 = nrm2(J, X + YY);
      rscal(J, 1 / SCLR1, X + YY);
    }
    gemv_n(N, J, T(1), X + VV, N, X + YY, T(0), X + UU);
    gemv_n(N, J, T(1), X + WW, N, X + YY, T(0), X + REIG);
    if (GEP) gemv_n(N, J, T(1), X + BV, N, X + YY, T(0), X + BU);
  } else {
    X[YY] = T(1);
    fillv(J - 1, T(0), X + YY + 1);
    copyv(N, X + VV, X + UU);
    copyv(N, X + WW, X + REIG);
    if (GEP) copyv(N, X + BV, X + BU);
  }
  if (GEP) NBU = nrm2(N, X + BU);
  if (ISERCH == 2) {
    if (GEP) {
      gemv_n(J, J, T(1), X + MM, MOD, X + YY, T(0), X + WL);
      THMT = re(dotc(J, X + WL, X + YY)) / (NBU * NBU);
    } else {
      hemv_u(J, X + MM, MOD, X + YY, X + WL);
      THMT = re(dotc(J, X + WL, X + YY));
    }
    THETA = THMT + SIGMA;
  } else {
    THMT = THETA;
    ETA0 = std::min(ETA0, THETA);
  }
  axpy(N, T(-THMT), X + BU, X + REIG);
  NREIGP = NREIG;
  NREIG = nrm2(N, X + REIG);
  if (GEP) NREIG /= NBU;
  if (neweig) { S.rinit = NREIG; neweig = false; }
  if (std::fabs(NREIG / NREIGP - 1) < 0.01) istag++;
  else istag = 0;
  if ((NREIG >= TOL && istag <= 2) || (NREIG >= TOL && RNDIND <= 1) || (NREIG >= TOL && RESID > 0.1 * NREIG))
    goto correction;
  // convergence detected in the extraction
  repgs(N, X + KXP, N, X + KBXP, N, NEIG, X + UU, X + WL, EPSM, 0);
  if (NEIG > 0 && X[WL + NEIG] == T(0)) goto err_orth;
  if (!GEP) {
    SCLR1 = (NEIG > 0) ? re(X[WL + NEIG]) : nrm2(N, X + UU);
  } else {
    bmatvec(UU, BU);
    if (!bnormalize(UU, BU, SCLR1)) goto err_bnotspd;
  }
  rscal(N, 1 / SCLR1, X + UU);

lock:  // label 18
  NEIG++;
  KXP = UU;
  KBXP = BU;
  UU -= N;
  BU -= N;
  EIGS[NWANT - NEIG] = THETA;
  RES[NWANT - NEIG] = NREIG;
  RINITM *= S.rinit;
  GAP = THETA2 - THETA;
  if (NEIG >= NWANT) goto finish;
  DELTA1 = RINF;
  NREIG = RINF;
  RESID = RINF;
  RNDIND = 0;
  if (ISERCH != 2) {
    ETA1 = std::min(ETA0, ETA1);
    for (int ii = 0; ii < NEIG; ++ii) ETA0 = std::max(ETA0, EIGS[ii]);
  }
  if (J == 1 || INITFLG) goto start_space;
  K = J;
  J = std::min(MIDSPACE + 1, J - 1);
  J = std::min(J, MOD - 1);
  if (ISERCH == 2)
    for (IJ = 2; IJ <= J + 1; ++IJ) repgs(K, X + YY, K, X + YY, K, 1, X + MP + MOD * (IJ - 1), X + WL, EPSM, 1);
  shrink(N, J, K, X + YY2, MOD, X + VV, X + WW, X + BV, X + MM, X + NN, MOD, ISERCH, GEP);
  UKNOWN = true;
  neweig = true;
  goto main_loop;

correction:  // label 20
  TRS = std::sqrt(1.0 / 10);
  if (istag > 0) TRS = 1.0 / 10;
  if (ITER >= MVMAX - NEIG - 1) goto err_maxit;
  if (J >= MOD) {
    K = J;
    J = MIDSPACE;
    shrink(N, J, K, X + MP, MOD, X + VV, X + WW, X + BV, X + MM, X + NN, MOD, ISERCH, GEP);
    SCLR1 = 0;
    long jj = 0;
    for (long i = 0; i < N; ++i)
      if (ab(X[UU + i]) > SCLR1) { SCLR1 = ab(X[UU + i]); jj = i; }
    AXPYALPHA = X[UU + jj] / X[VV + jj];
    X[YY] = AXPYALPHA / ab(AXPYALPHA);
    fillv(J - 1, T(0), X + YY + 1);
  }
  ETA = ETA0;
  if (J > 1) {
    DELTAO = DELTA1;
    if (ISERCH == 2) {
      if (GEP) {
        THETA2 = 1 / THETA2;
      } else {
        SCLR1 = nrm2(J, X + YY2);
        rscal(J, 1 / SCLR1, X + YY2);
        hemv_u(J, X + MM, MOD, X + YY2, X + WL);
        THETA2 = re(dotc(J, X + YY2, X + WL));
      }
      DELTA1 = std::fabs(THETA2) - std::fabs(THETA - SIGMA);
    } else {
      DELTA1 = THETA2 - THETA;
    }
    if (NREIG < std::fabs(DELTA1) && std::fabs(DELTA1 / DELTAO - 1) < 0.1) ETA = THETA;
  }
  repgs(N, X + BU, N, X + UU, N, NEIG + 1, X + REIG, X + WL, EPSM, -1);
  RNDIND = ab(X[WL + NEIG]) / (NREIG * EPSMSR);
  RESID = NREIG;
  {
    const long XCG = VV + J * N;
    int ITCG = MVMAX - ITER - NEIG - 1;
    IFO = (ISERCH != 2) ? 1 : 0;
    GK = RESID;
    S.rcurr = NREIG;
    if (NEIG <= 0) {
      S.shift1 = THETA;
      GAP = (J > 1) ? THETA2 - THETA : 0;
    }
    if (GEP) AXPYBETA = dotc(N, X + BU, X + REIG) / (NBU * NBU);
    // LSOLREVCOM: WORK columns R,Z,P,Q start at WCG (R aliases REIG, Z aliases WL)
    T* Xc = X + XCG;
    T *R = X + WCG, *Zv = X + WCG + N, *P = X + WCG + 2 * N, *Q = X + WCG + 3 * N;
    T* X2 = X + XCG2;
    T* BTv = X + BT;
    bool FTFLG = true;
    {
      const bool POSDEF = (IFO == 1);
      IFO = 0;
      const int MAXIT = ITCG;
      double GGK2 = GK * GK, RHO = 0, RHO1 = 0, TTK2 = 0, TTK2M = 0;
      if (POSDEF) fillv(N, T(0), Xc);
      if (GEP) fillv(N, T(0), BTv);
      int it = 0;
      bool fail = false;
      for (;;) {
        ++it;
        cb.precond(cb.ctx, R, Zv);  // IJOB=2 -> label 38
        S.flagcg = true;
        repgs(N, X + UU, N, X + BU, N, NEIG + 1, Zv, X + NP, EPSM, -1);
        RHO = re(dotc(N, R, Zv));
        if (POSDEF && RHO <= 0) {
          std::fprintf(stderr, " Non fatal bug: the preconditioner is not positive definite\n");
          fail = true;
          break;
        }
        if (RHO == 0) { fail = true; break; }
        if (it > 1) {
          axpy(N, T(RHO / RHO1), P, Zv);
          copyv(N, Zv, P);
        } else {
          copyv(N, Zv, P);
        }
        cb.matvec(cb.ctx, 1, P, Q, Zv);  // IJOB=1 -> label 37
        AXPYALPHA = T(-ETA);
        if (GEP) axpy(N, AXPYALPHA, Zv, Q);
        else axpy(N, AXPYALPHA, P, Q);
        if (GEP) AXPYALPHA = dotc(N, X + BU, Q) / (NBU * NBU);
        repgs(N, X + BU, N, X + UU, N, 1, Q, X + NP, EPSM, -1);
        ALPRHO = re(X[NP]);
        ITER++;
        alpha_cg = re(dotc(N, P, Q));
        if ((POSDEF && alpha_cg <= 0) || alpha_cg == 0) { fail = true; break; }
        alpha_cg = RHO / alpha_cg;
        axpy(N, T(-alpha_cg), Q, R);
        GK = nrm2(N, R);
        if (GEP) axpy(N, T(alpha_cg), Zv, BTv);
        if (POSDEF) {
          axpy(N, T(alpha_cg), P, Xc);
        } else {
          double GK2 = GK * GK;
          TTK2M = TTK2;
          TTK2 = GK2 / GGK2;
          double CK2 = 1 / (1 + TTK2);
          GGK2 = GGK2 * TTK2 * CK2;
          if (it > 1) {
            axpy(N, T(alpha_cg / TTK2M), P, X2);
            rscal(N, TTK2M * CK2, X2);
            axpy(N, T(1), X2, Xc);
          } else {
            copyv(N, P, X2);
            rscal(N, alpha_cg * CK2, X2);
            copyv(N, X2, Xc);
          }
        }
        // IJOB=3 -> label 33
        if (FTFLG) IFO = (ISERCH == 2) ? -2 : -1;
        AXPYALPHA *= alpha_cg;
        ALPRHO *= alpha_cg;
        stoptest(N, Xc, BTv, X + BU, TOL, RESID, NBU, ALPRHO, GK, AXPYALPHA, AXPYBETA, THETA, ETA, IFO, TRS, GEP);
        FTFLG = false;
        if (IFO == 1) { IFO = 0; break; }
        if (it == MAXIT) { fail = true; break; }
        RHO1 = RHO;
      }
      if (fail) {
        IFO = 1;
        if (alpha_cg <= 0) IFO = 2;
        if (it == 1) copyv(N, P, Xc);
      }
    }
    // label 34
    if (ISERCH != 2 && ETA <= ETA0 && NEIG > 0 && IFO == 2) ETA0 = std::min(ETA1, ETA0);
    CONV = false;
    S.flagcg = false;
    S.rcum += std::log(NREIG / RESID);
    if (RESID < TOL) {
      axpy(N, T(-1), Xc, X + UU);
      repgs(N, X + KXP, N, X + KBXP, N, NEIG, X + UU, X + NP, EPSM, 0);
      if (NEIG > 0 && X[NP + NEIG] == T(0)) goto err_orth;
      if (!GEP) {
        SCLR1 = (NEIG > 0) ? re(X[NP + NEIG]) : nrm2(N, X + UU);
      } else {
        bmatvec(UU, BU);
        if (!bnormalize(UU, BU, SCLR1)) goto err_bnotspd;
      }
      rscal(N, 1 / SCLR1, X + UU);
      THETA = THETA / SCLR1 + ETA;
      CONV = true;
      NREIG = RESID;
      if (NEIG >= NWANT - 1) goto lock;
    }
    // label 50: expand the search space with t
    repgs(N, X + KXP, N, X + KBXP, N, NEIG + J, Xc, X + REIG, EPSM, 1);
    axpy(J, T(-1), X + REIG + NEIG, X + YY);
    if (!GEP) {
      SCLR1 = re(X[REIG + NEIG + J]);
      rscal(N, 1 / SCLR1, Xc);
    }
    const long NDX2 = WW + J * N, NDX3 = BV + J * N;
    cb.matvec(cb.ctx, 1, Xc, X + NDX2, X + NDX3);
    ITER++;
    if (GEP) {
      SCLR1 = re(dotc(N, Xc, X + NDX3));
      if (SCLR1 <= 0) goto err_bnotspd;
      SCLR1 = std::sqrt(SCLR1);
      rscal(N, 1 / SCLR1, Xc);
      rscal(N, 1 / SCLR1, X + NDX2);
      rscal(N, 1 / SCLR1, X + NDX3);
    }
    X[YY + J] = T(-SCLR1);
    if (ISERCH == 2) axpy(N, T(-SIGMA), X + NDX3, X + NDX2);
    if (ISERCH == 2 && GEP) {
      gemv_c(N, J + 1, T(1), X + WW, N, X + NDX3, T(0), X + MM + J * MOD);
      for (long r = 0; r < J; ++r) X[MM + J + r * MOD] = cj(dotc(N, X + BV + r * N, X + NDX2));
    } else {
      gemv_c(N, J + 1, T(1), X + VV, N, X + NDX2, T(0), X + MM + J * MOD);
    }
    if (ISERCH == 2) gemv_c(N, J + 1, T(1), X + WW, N, X + NDX2, T(0), X + NN + J * MOD);
    J++;
    UKNOWN = false;
    if (!CONV) goto main_loop;
  }
  // convergence inside the inner solve: deflate the converged direction
  if (ISERCH != 2 || !GEP) {
    SCLR1 = nrm2(J, X + YY);
    rscal(J, 1 / SCLR1, X + YY);
  }
  if (ISERCH == 2) {
    hemv_u(J, X + NN, MOD, X + YY, X + WL2);
    SCLR1 = re(dotc(J, X + YY, X + WL2));
    if (GEP) {
      gemv_n(J, J, T(1), X + MM, MOD, X + YY, T(0), X + WL);
      AXPYALPHA = dotc(J, X + YY, X + WL);
      THMT = re(AXPYALPHA) / (ALPRHO * NBU * NBU);
      AXPYALPHA = -AXPYALPHA / SCLR1;
      axpy(J, AXPYALPHA, X + WL2, X + WL);
      gemv_c(J, J, T(1), X + MM, MOD, X + YY, T(0), X + WL3);
      copyv(MOD * MOD, X + MM, X + MP);
      for (long c = 0; c < J; ++c)
        for (long r = 0; r < J; ++r)
          X[MP + r + c * MOD] += T(-1 / SCLR1) * (X[WL + r] * cj(X[WL2 + c]) + X[WL2 + r] * cj(X[WL3 + c]));
    } else {
      hemv_u(J, X + MM, MOD, X + YY, X + WL);
      THMT = re(dotc(J, X + YY, X + WL));
      axpy(J, T(-THMT / (2 * SCLR1)), X + WL2, X + WL);
      T al = T(-1 / SCLR1);
      copyv(MOD * MOD, X + MM, X + MP);
      for (long c = 0; c < J; ++c)  // SYR2 upper: al x y^H + conj(al) y x^H
        for (long r = 0; r <= c; ++r)
          X[MP + r + c * MOD] += al * X[WL + r] * cj(X[WL2 + c]) + cj(al) * X[WL2 + r] * cj(X[WL + c]);
    }
    THETA = THMT + SIGMA;
    copyv(MOD * MOD, X + NN, X + NP);
  } else {
    hemv_u(J, X + MM, MOD, X + YY, X + WL);
    THETA = re(dotc(J, X + YY, X + WL));
    ETA0 = std::min(ETA0, THETA);
    SCLR1 = 0;
    for (long i = 0; i < J; ++i) SCLR1 += ab2(X[MP + i * (MOD + 1)]);
    SCLR1 = std::sqrt(SCLR1);
    if (THETA < 0) SCLR1 -= 2 * THETA;
    axpy(J, T(SCLR1), X + YY, X + WL);
    copyv(J, X + YY, X + WL2);
    copyv(MOD * MOD, X + MM, X + MP);
    for (long c = 0; c < J; ++c)
      for (long r = 0; r <= c; ++r)
        X[MP + r + c * MOD] += T(-1) * X[WL2 + r] * cj(X[WL + c]) + T(-1) * X[WL + r] * cj(X[WL2 + c]);
  }
  solprojep(J, X + MP, X + NP, MOD, SCLR1, SCLR2, Wr, -ISERCH, INFO, GEP);
  if (INFO != 0) goto err_lapack;
  if (ISERCH == 2) {
    SCLR1 = nrm2(J, X + YY);
    rscal(J, 1 / SCLR1, X + YY);
  }
  goto lock;

err_lapack:
  if (INFO > 0) INFO = -INFO;
  goto abnormal;
err_orth:
  INFO = -54320;
  goto abnormal;
err_bnotspd:
  INFO = -54322;
  goto abnormal;
err_maxit:
  INFO = NEIG + 1;
  RINITM *= S.rinit;
abnormal:  // label 198
  if (NEIG > 0) copyv(N, X + UU, X + VV);
  if (NEIG > 0 && GEP) copyv(N, X + BU, X + BV);

finish:  // label 200
{
  if (NEIG < NWANT) {
    S.rinit = std::pow(RINITM, 1.0 / (NEIG + 1));
    if (NEIG > 0) {
      long jj = std::min<long>(NEIG, NWANT - NEIG);
      copyv(N * jj, X + N * (NWANT - jj) + XX, X + XX);
      for (long i = 0; i < jj; ++i) { EIGS[i] = EIGS[NWANT - jj + i]; RES[i] = RES[NWANT - jj + i]; }
      copyv(N, X + VV, X + N * NEIG + XX);
      if (GEP) {
        copyv(N * jj, X + N * (NWANT - jj) + BX, X + BX);
        copyv(N, X + BV, X + N * NEIG + BX);
      }
      EIGS[NEIG] = THETA;
      RES[NEIG] = NREIG;
      THETA2 = THETA;
    } else {
      copyv(N, X + UU, X + XX);
      if (GEP) copyv(N, X + BU, X + BX);
      EIGS[0] = THETA;
      RES[0] = NREIG;
      GAP = 0;
      return;
    }
  } else {
    S.rinit = std::pow(RINITM, 1.0 / NEIG);
  }
  sortev(N, NEIG, X + XX, N, X + BX, N, EIGS, RES, GEP ? -4 : 4, 0.0);
  long ITARG = 0;
  if (ISERCH >= 2) {
    for (ITARG = 1; ITARG <= NEIG; ++ITARG)
      if (EIGS[ITARG - 1] > SIGMA) break;
  }
  if (ISERCH == 2) GAP = std::fabs(THETA2 - SIGMA) - std::max(std::fabs(EIGS[NEIG - 1] - SIGMA), std::fabs(EIGS[0] - SIGMA));
  else GAP = THETA2 - EIGS[NEIG - 1];
  double GG = (ISERCH == 2) ? EIGS[0] + EIGS[NEIG - 1] - 2 * SIGMA : RINF;
  long II, JJ;
  if (GG > 0) { II = 1; JJ = NEIG - 1; }
  else { II = 2; JJ = NEIG; }
  if (NEIG == 1) { II = 0; JJ = 0; }
  auto E = [&](long i) -> double& { return EIGS[i - 1]; };  // 1-based views
  auto Rr = [&](long i) -> double& { return RES[i - 1]; };
  long I = 1;
  double GL = 0, GR = 0;
  while (I <= NEIG) {
    bool cluster = false;
    long Jc = 0;
    if (!(I < II || I >= JJ)) {
      GL = (I == 1) ? GG - Rr(NEIG) : E(I) - E(I - 1) - Rr(I - 1);
      if (!(GL < 10 * (E(I + 1) - E(I)))) {
        long Jx = std::min(I + MOD, JJ + 1);
        for (;;) {
          Jx--;
          if (Jx == I) break;
          GR = (Jx == NEIG) ? -GG - Rr(1) : E(Jx + 1) - E(Jx) - Rr(Jx + 1);
          if (!(10 * (E(Jx) - E(I)) > std::min(GL, GR))) { cluster = true; Jc = Jx - I + 1; break; }
        }
      }
    }
    if (cluster) {
      copyv(N * Jc, X + N * (I - 1) + XX, X + VV);
      for (long ij = 0; ij < Jc; ++ij) {
        cb.matvec(cb.ctx, 3, X + VV + ij * N, X + WW + ij * N, nullptr);
        ITER++;
      }
      for (long c = 0; c < Jc; ++c)
        for (long r = 0; r <= c; ++r)
          X[MM + r + c * MOD] = 0.5 * (dotc(N, X + VV + r * N, X + WW + c * N) + dotc(N, X + WW + r * N, X + VV + c * N));
      int inf2 = 0;
      solprojep(Jc, X + MM, X + NP, MOD, SCLR1, SCLR2, Wr, 3, inf2, GEP);
      if (inf2 == 0) {
        std::vector<T> tmp((size_t)N * Jc);
        auto blk = [&](long src, long dst) {  // X(dst) = X(src) * MM(1:Jc,1:Jc)
          for (long c = 0; c < Jc; ++c) gemv_n(N, Jc, T(1), X + src, N, X + MM + c * MOD, T(0), tmp.data() + c * N);
          copyv(N * Jc, tmp.data(), X + dst);
        };
        blk(VV, N * (I - 1) + XX);
        blk(WW, VV);
        if (GEP) {
          copyv(N * Jc, X + N * (I - 1) + BX, X + BV);
          blk(BV, N * (I - 1) + BX);
        }
        double NRC = 0;
        GL -= E(I);
        GR += E(I + Jc - 1);
        for (long ij = 1; ij <= Jc; ++ij) {
          double th = re(X[NP + ij - 1]);
          E(I + ij - 1) = th;
          axpy(N, T(-th), X + N * (I + ij - 2) + BX, X + VV + N * (ij - 1));
          double nr = nrm2(N, X + VV + N * (ij - 1));
          if (GEP) nr /= nrm2(N, X + N * (I + ij - 2) + BX);
          Rr(I + ij - 1) = nr;
          NRC += nr * nr;
        }
        for (long ij = I; ij <= I + Jc - 1; ++ij)
          if (ij == ITARG) ITARG--;
        I += Jc;
        continue;
      }
    }
    // label 250: isolated eigenvalue, true residual
    cb.matvec(cb.ctx, 3, X + N * (I - 1), X + VV, nullptr);
    ITER++;
    {
      double th = re(dotc(N, X + N * (I - 1) + XX, X + VV));
      axpy(N, T(-th), X + N * (I - 1) + BX, X + VV);
      double nr = nrm2(N, X + VV);
      if (GEP) nr /= nrm2(N, X + N * (I - 1) + BX);
      E(I) = th;
      Rr(I) = nr;
      if (I == ITARG) ITARG--;
    }
    I++;
  }
}
}

}  // namespace orc
