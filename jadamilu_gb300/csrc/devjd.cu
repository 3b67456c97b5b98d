// Jacobi-Davidson core on device vectors: the outer loop of JDRVCOM
// (src/jd/JDaux.F:1391-2415), the inner CG / smoothed-CG solve of LSOLREVCOM
// (:2989-3268) and STOPTEST (:2542-2672).  See devjd.cuh for the data layout.
#include "devjd.cuh"

namespace jdg {

template <class T>
void DevJd<T>::stoptest(long N, long x, long bt, long bu, double tol, double& rk, double nbu, double& alprho,
                        double& gk, H pcad, H pcr, double& theta, double eta, int& info, double trs, bool gep) {
  StopStateD<T>& s = st;
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
    if (gep) s.bkgep = H(theta - eta) + pcr;
    s.un2 = -1;
  }
  s.bk -= alprho;
  if (gep) {
    s.bkgep -= pcad;
    s.beta = habs(s.bkgep);
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
          s.bubt = -dot(N, bu, bt) / (nbu * nbu);
          s.alp = habs(H(1) + s.bubt);
          s.tn = std::sqrt(hre(jdd::cj(H(s.tn) + s.bubt) * (H(s.tn) - s.bubt))) / s.alp;
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

// REPGS on small host vectors (restart of the harmonic extraction)
template <class H> static void repgs_small(long N, const H* V, long JV, H* w, H* y, double epsm, Lcg48d& rng) {
  bool nrnd = true;
  if (JV <= 0) return;
  for (;;) {
    double nrn = jdd::nrm2(N, w), nr = epsm * nrn, nro;
    if (nrnd) jdd::fillv(JV, H(0), y);
    bool small = false;
    do {
      nro = nrn;
      jdd::gemv_c(N, JV, H(1), V, N, w, H(0), y + JV);
      jdd::gemv_n(N, JV, H(-1), V, N, y + JV, H(1), w);
      nrn = jdd::nrm2(N, w);
      if (nrnd) jdd::axpy(JV, H(1), y + JV, y);
      if (nrn <= nr) { small = true; break; }
    } while (nrn < 0.5 * nro);
    if (!small) { y[JV] = H(nrn); return; }
    if (JV < N) {
      for (long i = 0; i < N; ++i) w[i] = H(rng.next());
      nrnd = false;
      continue;
    }
    return;
  }
}

template <class T>
void DevJd<T>::run(long N, double* EIGS, double* RES, int LXi, int& NEIG, double SIGMA, int ISEARCH, int NINIT,
                   int MADSPACE, int& ITER, double TOL, int& INFO, double& GAP, bool GEP) {
  const long LX = LXi;
  const double EPSM = DBL_EPSILON * 0.5, RINF = DBL_MAX;
  JdState& S_ = *sh;
  S_.flagcg = true;
  bool neweig = true;
  S_.rcum = 0;
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
  if (MOD > 32) throw std::runtime_error("MADSPACE above 32 is not supported by the GPU restart kernel");
  const int MVMAX = ITER;
  int ISERCH = std::min(ISEARCH, 2);
  const long XX = 0, VV = XX + NWANT * N, WW = VV + MOD * N;
  long BX, BV, MM;
  if (GEP) { BX = WW + MOD * N; BV = BX + NWANT * N; MM = BV + MOD * N; }
  else { BX = XX; BV = VV; MM = WW + MOD * N; }
  const long NN = MM + MOD * MOD, MP = NN + MOD * MOD, NP = MP + MOD * MOD;
  const long WCG = NP + std::max(MOD * MOD, NWANT);
  const long XCG2 = WW + (MOD - 1) * N, BT = BV + (MOD - 1) * N, REIG = WCG, YY = MP, YY2 = MP + MOD;
  const long WL = REIG + N, WL2 = WL + MOD, WL3 = WL2 + MOD;
  long UU = XX + (NWANT - 1) * N, BU = BX + (NWANT - 1) * N, KXP = VV, KBXP = BV;
  H* X = hX;  // host side of the workspace (small arrays)
  double* Wr = reinterpret_cast<double*>(X + REIG);
  const double EPSMSR = std::sqrt(EPSM);
  NEIG = 0;
  ITER = 0;
  double ETA1 = RINF, ETA0 = SIGMA, DELTA1 = RINF, NREIG = RINF, RESID = RINF, RNDIND = 0, DELTAO = 0;
  if (ISERCH == 0) ETA0 = RINF;
  const long MIDSPACE = (MOD + 1) / 2;
  bool INITFLG = false, UKNOWN = false, CONV = false;
  double THETA = 0, THETA2 = 0, THMT = 0, NBU = 1, NREIGP = 0, TRS = 0, ETA = 0, SCLR1 = 0, SCLR2 = 0, ALPRHO = 0,
         GK = 0;
  H AXPYALPHA = H(0), AXPYBETA = H(0);
  long J = 0, K = 0, IJ = 0;
  int IFO = 0;
  int istep = 0;
  std::vector<H> t1(2 * MOD + 8), t2(2 * MOD + 8);
  if (NINIT > MIDSPACE) {
    for (int ii = 1; ii < NINIT; ++ii)
      if (EIGS[ii] != EIGS[0]) INITFLG = true;
    if (INITFLG) {
      if (NINIT > 32) throw std::runtime_error("NINIT above 32");
      sortev_dev(N, NINIT, XX, XX, EIGS, RES, ISERCH, SIGMA);
    } else {
      for (int ii = 0; ii < NINIT / 2; ++ii) {
        int jj = NINIT - 1 - ii;
        copy(N, (long)jj * N, VV);
        copy(N, (long)ii * N, (long)jj * N);
        copy(N, VV, (long)ii * N);
      }
    }
  }
  INITFLG = false;

  auto bnormalize = [&](long u, long bu, double& s) -> bool {
    s = hre(dot(N, u, bu));
    if (s <= 0) return false;
    s = std::sqrt(s);
    scal(N, 1 / s, bu);
    return true;
  };

start_space:
  if (NINIT <= NEIG) {
    J = 1;
    fill(N, H(1), VV);
  } else {
    J = std::min<long>(NINIT - NEIG, MIDSPACE);
    IJ = NINIT - NEIG - J;
    if (IJ > 0) INITFLG = true;
    copy(N * J, N * IJ, VV);
  }
  for (IJ = 1; IJ <= J; ++IJ) {
    long vj = VV + (IJ - 1) * N;
    repgs(N, KXP, KBXP, NEIG + IJ - 1, vj, X + WL, EPSM, 1);
    if (!GEP) {
      SCLR1 = (NEIG + IJ - 1 > 0) ? hre(X[WL + NEIG + IJ - 1]) : nrm2(N, VV);
      scal(N, 1 / SCLR1, vj);
    }
    matvec(1, vj, WW + (IJ - 1) * N, BV + (IJ - 1) * N);
    ITER++;
    if (GEP) {
      long bvj = BV + (IJ - 1) * N;
      SCLR1 = hre(dot(N, vj, bvj));
      if (SCLR1 <= 0) goto err_bnotspd;
      SCLR1 = std::sqrt(SCLR1);
      scal(N, 1 / SCLR1, bvj);
      scal(N, 1 / SCLR1, vj);
      scal(N, 1 / SCLR1, WW + (IJ - 1) * N);
    }
  }
  if (ISERCH == 2) {
    axpy(N * J, H(-SIGMA), BV, WW);
    for (long c = 0; c < J; ++c) gemvc(N, (int)c + 1, WW, N, WW + c * N, X + NN + c * MOD);
  }
  if (ISERCH == 2 && GEP) {
    for (long c = 0; c < J; ++c) gemvc(N, (int)J, WW, N, BV + c * N, X + MM + c * MOD);
  } else {
    for (long c = 0; c < J; ++c) {
      gemvc(N, (int)c + 1, VV, N, WW + c * N, t1.data());
      gemvc(N, (int)c + 1, WW, N, VV + c * N, t2.data());
      for (long r = 0; r <= c; ++r) X[MM + r + c * MOD] = t1[r] + t2[r];
    }
    jdd::rscal(MOD * MOD, 0.5, X + MM);
  }
  UKNOWN = (J <= 1);

main_loop:
  jdd::copyv(MOD * MOD, X + MM, X + MP);
  if (ISERCH == 2) jdd::copyv(MOD * MOD, X + NN, X + NP);
  solprojep(J, X + MP, X + NP, MOD, THETA, THETA2, Wr, ISERCH, INFO, GEP);
  if (INFO != 0) goto err_lapack;
  if (!UKNOWN) {
    if (ISERCH == 2) {
      SCLR1 = jdd::nrm2(J, X + YY);
      jdd::rscal(J, 1 / SCLR1, X + YY);
    }
    gemvn(N, (int)J, H(1), VV, N, X + YY, H(0), UU);
    gemvn(N, (int)J, H(1), WW, N, X + YY, H(0), REIG);
    if (GEP) gemvn(N, (int)J, H(1), BV, N, X + YY, H(0), BU);
  } else {
    X[YY] = H(1);
    jdd::fillv(J - 1, H(0), X + YY + 1);
    copy(N, VV, UU);
    copy(N, WW, REIG);
    if (GEP) copy(N, BV, BU);
  }
  if (GEP) NBU = nrm2(N, BU);
  if (ISERCH == 2) {
    if (GEP) {
      jdd::gemv_n(J, J, H(1), X + MM, MOD, X + YY, H(0), X + WL);
      THMT = hre(jdd::dotc(J, X + WL, X + YY)) / (NBU * NBU);
    } else {
      jdd::hemv_u(J, X + MM, MOD, X + YY, X + WL);
      THMT = hre(jdd::dotc(J, X + WL, X + YY));
    }
    THETA = THMT + SIGMA;
  } else {
    THMT = THETA;
    ETA0 = std::min(ETA0, THETA);
  }
  axpy(N, H(-THMT), BU, REIG);
  NREIGP = NREIG;
  NREIG = nrm2(N, REIG);
  if (GEP) NREIG /= NBU;
  if (neweig) { S_.rinit = NREIG; neweig = false; }
  if (std::fabs(NREIG / NREIGP - 1) < 0.01) istag++;
  else istag = 0;
  if ((NREIG >= TOL && istag <= 2) || (NREIG >= TOL && RNDIND <= 1) || (NREIG >= TOL && RESID > 0.1 * NREIG))
    goto correction;
  repgs(N, KXP, KBXP, NEIG, UU, X + WL, EPSM, 0);
  if (NEIG > 0 && X[WL + NEIG] == H(0)) goto err_orth;
  if (!GEP) {
    SCLR1 = (NEIG > 0) ? hre(X[WL + NEIG]) : nrm2(N, UU);
  } else {
    matvec(4, UU, -1, BU);
    if (!bnormalize(UU, BU, SCLR1)) goto err_bnotspd;
  }
  scal(N, 1 / SCLR1, UU);

lock:
  NEIG++;
  KXP = UU;
  KBXP = BU;
  UU -= N;
  BU -= N;
  EIGS[NWANT - NEIG] = THETA;
  RES[NWANT - NEIG] = NREIG;
  RINITM *= S_.rinit;
  if (on_step) on_step(1, istep, NEIG, THETA, (double)ITER);
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
    for (IJ = 2; IJ <= J + 1; ++IJ) repgs_small(K, X + YY, 1, X + MP + MOD * (IJ - 1), X + WL, EPSM, rng);
  shrink(N, J, K, X + YY2, MOD, VV, WW, BV, X + MM, X + NN, MOD, ISERCH, GEP);
  UKNOWN = true;
  neweig = true;
  goto main_loop;

correction:
  if (on_step) on_step(0, istep, NEIG + 1, THETA, NREIG);
  TRS = std::sqrt(1.0 / 10);
  if (istag > 0) TRS = 1.0 / 10;
  istep++;
  if (ITER >= MVMAX - NEIG - 1) goto err_maxit;
  if (J >= MOD) {
    K = J;
    J = MIDSPACE;
    shrink(N, J, K, X + MP, MOD, VV, WW, BV, X + MM, X + NN, MOD, ISERCH, GEP);
    // first index of the largest |u_i|, then the phase of u relative to the new V(:,1)
    std::vector<T> hu(N);
    CK(cudaMemcpyAsync(hu.data(), D(UU), sizeof(T) * N, cudaMemcpyDeviceToHost, S()));
    sync();
    SCLR1 = 0;
    long jj = 0;
    for (long i = 0; i < N; ++i) {
      double a = std::sqrt(ab2(hu[i]));
      if (a > SCLR1) { SCLR1 = a; jj = i; }
    }
    T uj = hu[jj], vj;
    CK(cudaMemcpyAsync(&vj, D(VV + jj), sizeof(T), cudaMemcpyDeviceToHost, S()));
    sync();
    H ujh = reinterpret_cast<H&>(uj), vjh = reinterpret_cast<H&>(vj);
    AXPYALPHA = ujh / vjh;
    X[YY] = AXPYALPHA / habs(AXPYALPHA);
    jdd::fillv(J - 1, H(0), X + YY + 1);
  }
  ETA = ETA0;
  if (J > 1) {
    DELTAO = DELTA1;
    if (ISERCH == 2) {
      if (GEP) {
        THETA2 = 1 / THETA2;
      } else {
        SCLR1 = jdd::nrm2(J, X + YY2);
        jdd::rscal(J, 1 / SCLR1, X + YY2);
        jdd::hemv_u(J, X + MM, MOD, X + YY2, X + WL);
        THETA2 = hre(jdd::dotc(J, X + YY2, X + WL));
      }
      DELTA1 = std::fabs(THETA2) - std::fabs(THETA - SIGMA);
    } else {
      DELTA1 = THETA2 - THETA;
    }
    if (NREIG < std::fabs(DELTA1) && std::fabs(DELTA1 / DELTAO - 1) < 0.1) ETA = THETA;
  }
  repgs(N, BU, UU, NEIG + 1, REIG, X + WL, EPSM, -1);
  RNDIND = habs(X[WL + NEIG]) / (NREIG * EPSMSR);
  RESID = NREIG;
  {
    const long XCG = VV + J * N;
    int ITCG = MVMAX - ITER - NEIG - 1;
    IFO = (ISERCH != 2) ? 1 : 0;
    GK = RESID;
    S_.rcurr = NREIG;
    if (NEIG <= 0) {
      S_.shift1 = THETA;
      GAP = (J > 1) ? THETA2 - THETA : 0;
    }
    if (GEP) AXPYBETA = dot(N, BU, REIG) / (NBU * NBU);
    const long R = WCG, Zv = WCG + N, P = WCG + 2 * N, Q = WCG + 3 * N, X2 = XCG2, BTv = BT, Xc = XCG;
    bool FTFLG = true;
    {
      const bool POSDEF = (IFO == 1);
      IFO = 0;
      const int MAXIT = ITCG;
      double GGK2 = GK * GK, RHO = 0, RHO1 = 0, TTK2 = 0, TTK2M = 0;
      if (POSDEF) fill(N, H(0), Xc);
      if (GEP) fill(N, H(0), BTv);
      int it = 0;
      bool fail = false;
      // RHO of iteration `it` is kept in device slot kScal + (it & 1), so the
      // next iteration finds its predecessor there.
      T* const scd = W->dsm + kScal;
      for (;;) {
        ++it;
        if (device_ops && it > 1) {
          // The same operations in the same order, with RHO, the projection
          // coefficient, P^H Q, B-inner product and |R|^2 left on the
          // device and read back together: one synchronisation per
          // iteration.  The checks on RHO and P^H Q come after the read;
          // a failed check leaves P, Q, Z and R modified where the plain
          // sequence stops earlier, and none of them is read after a failed
          // inner solve (it > 1).
          precond(R, Zv);
          S_.flagcg = true;
          repgs(N, UU, BU, NEIG + 1, Zv, nullptr, EPSM, -1);
          T* rho_d = scd + (it & 1);
          k::mdot<T>(N, 1, D(R), N, D(Zv), rho_d, W->dpart, S());
          k::axpy_ratio_copy<T>(N, rho_d, scd + ((it - 1) & 1), D(P), D(Zv), D(P), S());
          AXPYALPHA = H(-ETA);
          if (!GEP && matvec_shift) {
            matvec_shift(P, Q, AXPYALPHA);
          } else {
            matvec(1, P, Q, Zv);
            if (GEP) axpy(N, AXPYALPHA, Zv, Q);
            else axpy(N, AXPYALPHA, P, Q);
          }
          if (GEP) k::mdot<T>(N, 1, D(BU), N, D(Q), scd + 4, W->dpart, S());
          cgs_dev(N, BU, UU, 1, Q, scd + 2);
          k::mdot<T>(N, 1, D(P), N, D(Q), scd + 3, W->dpart, S());
          k::axpy_ratio<T>(N, rho_d, scd + 3, -1.0, D(Q), D(R), S());
          k::mdot<T>(N, 1, D(R), N, D(R), scd + 5, W->dpart, S());
          CK(cudaMemcpyAsync(W->hsm + kScal, scd, sizeof(T) * 6, cudaMemcpyDeviceToHost, S()));
          sync();
          const H* hs = reinterpret_cast<const H*>(W->hsm + kScal);
          RHO = hre(hs[it & 1]);
          if (POSDEF && RHO <= 0) {
            std::fprintf(stderr, " Non fatal bug: the preconditioner is not positive definite\n");
            fail = true;
            break;
          }
          if (RHO == 0) { fail = true; break; }
          if (GEP) AXPYALPHA = hs[4] / (NBU * NBU);
          X[NP] = hs[2];
          ALPRHO = hre(X[NP]);
          ITER++;
          alpha_cg = hre(hs[3]);
          if ((POSDEF && alpha_cg <= 0) || alpha_cg == 0) { fail = true; break; }
          alpha_cg = RHO / alpha_cg;
          GK = std::sqrt(rl(W->hsm[kScal + 5]));
        } else {
        precond(R, Zv);
        S_.flagcg = true;
        repgs(N, UU, BU, NEIG + 1, Zv, nullptr, EPSM, -1);
        k::mdot<T>(N, 1, D(R), N, D(Zv), scd + (it & 1), W->dpart, S());
        CK(cudaMemcpyAsync(W->hsm + kScal, scd + (it & 1), sizeof(T), cudaMemcpyDeviceToHost, S()));
        sync();
        RHO = hre(reinterpret_cast<const H*>(W->hsm + kScal)[0]);
        if (POSDEF && RHO <= 0) {
          std::fprintf(stderr, " Non fatal bug: the preconditioner is not positive definite\n");
          fail = true;
          break;
        }
        if (RHO == 0) { fail = true; break; }
        if (it > 1) {
          axpy(N, H(RHO / RHO1), P, Zv);
          copy(N, Zv, P);
        } else {
          copy(N, Zv, P);
        }
        matvec(1, P, Q, Zv);
        AXPYALPHA = H(-ETA);
        if (GEP) axpy(N, AXPYALPHA, Zv, Q);
        else axpy(N, AXPYALPHA, P, Q);
        if (GEP) AXPYALPHA = dot(N, BU, Q) / (NBU * NBU);
        repgs(N, BU, UU, 1, Q, X + NP, EPSM, -1);
        ALPRHO = hre(X[NP]);
        ITER++;
        alpha_cg = hre(dot(N, P, Q));
        if ((POSDEF && alpha_cg <= 0) || alpha_cg == 0) { fail = true; break; }
        alpha_cg = RHO / alpha_cg;
        axpy(N, H(-alpha_cg), Q, R);
        GK = nrm2(N, R);
        }
        if (GEP) axpy(N, H(alpha_cg), Zv, BTv);
        if (POSDEF) {
          axpy(N, H(alpha_cg), P, Xc);
        } else {
          double GK2 = GK * GK;
          TTK2M = TTK2;
          TTK2 = GK2 / GGK2;
          double CK2 = 1 / (1 + TTK2);
          GGK2 = GGK2 * TTK2 * CK2;
          if (it > 1) {
            k::smooth<T>(N, todev(H(alpha_cg / TTK2M)), D(P), TTK2M * CK2, D(X2), D(Xc), S());
          } else {
            copy(N, P, X2);
            scal(N, alpha_cg * CK2, X2);
            copy(N, X2, Xc);
          }
        }
        if (FTFLG) IFO = (ISERCH == 2) ? -2 : -1;
        AXPYALPHA *= alpha_cg;
        ALPRHO *= alpha_cg;
        stoptest(N, Xc, BTv, BU, TOL, RESID, NBU, ALPRHO, GK, AXPYALPHA, AXPYBETA, THETA, ETA, IFO, TRS, GEP);
        FTFLG = false;
        if (IFO == 1) { IFO = 0; break; }
        if (it == MAXIT) { fail = true; break; }
        RHO1 = RHO;
      }
      if (fail) {
        IFO = 1;
        if (alpha_cg <= 0) IFO = 2;
        if (it == 1) copy(N, P, Xc);
      }
    }
    if (ISERCH != 2 && ETA <= ETA0 && NEIG > 0 && IFO == 2) ETA0 = std::min(ETA1, ETA0);
    CONV = false;
    S_.flagcg = false;
    S_.rcum += std::log(NREIG / RESID);
    if (RESID < TOL) {
      axpy(N, H(-1), Xc, UU);
      repgs(N, KXP, KBXP, NEIG, UU, X + NP, EPSM, 0);
      if (NEIG > 0 && X[NP + NEIG] == H(0)) goto err_orth;
      if (!GEP) {
        SCLR1 = (NEIG > 0) ? hre(X[NP + NEIG]) : nrm2(N, UU);
      } else {
        matvec(4, UU, -1, BU);
        if (!bnormalize(UU, BU, SCLR1)) goto err_bnotspd;
      }
      scal(N, 1 / SCLR1, UU);
      THETA = THETA / SCLR1 + ETA;
      CONV = true;
      NREIG = RESID;
      if (NEIG >= NWANT - 1) goto lock;
    }
    repgs(N, KXP, KBXP, NEIG + J, Xc, X + REIG, EPSM, 1);
    jdd::axpy(J, H(-1), X + REIG + NEIG, X + YY);
    if (!GEP) {
      SCLR1 = hre(X[REIG + NEIG + J]);
      scal(N, 1 / SCLR1, Xc);
    }
    const long NDX2 = WW + J * N, NDX3 = BV + J * N;
    matvec(1, Xc, NDX2, NDX3);
    ITER++;
    if (GEP) {
      SCLR1 = hre(dot(N, Xc, NDX3));
      if (SCLR1 <= 0) goto err_bnotspd;
      SCLR1 = std::sqrt(SCLR1);
      scal(N, 1 / SCLR1, Xc);
      scal(N, 1 / SCLR1, NDX2);
      scal(N, 1 / SCLR1, NDX3);
    }
    X[YY + J] = H(-SCLR1);
    if (ISERCH == 2) axpy(N, H(-SIGMA), NDX3, NDX2);
    if (ISERCH == 2 && GEP) {
      gemvc(N, (int)J + 1, WW, N, NDX3, X + MM + J * MOD);
      gemvc(N, (int)J, BV, N, NDX2, t1.data());
      for (long r = 0; r < J; ++r) X[MM + J + r * MOD] = jdd::cj(t1[r]);
    } else {
      gemvc(N, (int)J + 1, VV, N, NDX2, X + MM + J * MOD);
    }
    if (ISERCH == 2) gemvc(N, (int)J + 1, WW, N, NDX2, X + NN + J * MOD);
    J++;
    UKNOWN = false;
    if (!CONV) goto main_loop;
  }
  if (ISERCH != 2 || !GEP) {
    SCLR1 = jdd::nrm2(J, X + YY);
    jdd::rscal(J, 1 / SCLR1, X + YY);
  }
  if (ISERCH == 2) {
    jdd::hemv_u(J, X + NN, MOD, X + YY, X + WL2);
    SCLR1 = hre(jdd::dotc(J, X + YY, X + WL2));
    if (GEP) {
      jdd::gemv_n(J, J, H(1), X + MM, MOD, X + YY, H(0), X + WL);
      AXPYALPHA = jdd::dotc(J, X + YY, X + WL);
      THMT = hre(AXPYALPHA) / (ALPRHO * NBU * NBU);
      AXPYALPHA = -AXPYALPHA / SCLR1;
      jdd::axpy(J, AXPYALPHA, X + WL2, X + WL);
      jdd::gemv_c(J, J, H(1), X + MM, MOD, X + YY, H(0), X + WL3);
      jdd::copyv(MOD * MOD, X + MM, X + MP);
      for (long c = 0; c < J; ++c)
        for (long r = 0; r < J; ++r)
          X[MP + r + c * MOD] += H(-1 / SCLR1) * (X[WL + r] * jdd::cj(X[WL2 + c]) + X[WL2 + r] * jdd::cj(X[WL3 + c]));
    } else {
      jdd::hemv_u(J, X + MM, MOD, X + YY, X + WL);
      THMT = hre(jdd::dotc(J, X + YY, X + WL));
      jdd::axpy(J, H(-THMT / (2 * SCLR1)), X + WL2, X + WL);
      H al = H(-1 / SCLR1);
      jdd::copyv(MOD * MOD, X + MM, X + MP);
      for (long c = 0; c < J; ++c)
        for (long r = 0; r <= c; ++r)
          X[MP + r + c * MOD] += al * X[WL + r] * jdd::cj(X[WL2 + c]) + jdd::cj(al) * X[WL2 + r] * jdd::cj(X[WL + c]);
    }
    THETA = THMT + SIGMA;
    jdd::copyv(MOD * MOD, X + NN, X + NP);
  } else {
    jdd::hemv_u(J, X + MM, MOD, X + YY, X + WL);
    THETA = hre(jdd::dotc(J, X + YY, X + WL));
    ETA0 = std::min(ETA0, THETA);
    SCLR1 = 0;
    for (long i = 0; i < J; ++i) SCLR1 += jdd::ab2(X[MP + i * (MOD + 1)]);
    SCLR1 = std::sqrt(SCLR1);
    if (THETA < 0) SCLR1 -= 2 * THETA;
    jdd::axpy(J, H(SCLR1), X + YY, X + WL);
    jdd::copyv(J, X + YY, X + WL2);
    jdd::copyv(MOD * MOD, X + MM, X + MP);
    for (long c = 0; c < J; ++c)
      for (long r = 0; r <= c; ++r)
        X[MP + r + c * MOD] += H(-1) * X[WL2 + r] * jdd::cj(X[WL + c]) + H(-1) * X[WL + r] * jdd::cj(X[WL2 + c]);
  }
  solprojep(J, X + MP, X + NP, MOD, SCLR1, SCLR2, Wr, -ISERCH, INFO, GEP);
  if (INFO != 0) goto err_lapack;
  if (ISERCH == 2) {
    SCLR1 = jdd::nrm2(J, X + YY);
    jdd::rscal(J, 1 / SCLR1, X + YY);
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
  RINITM *= S_.rinit;
abnormal:
  if (NEIG > 0) copy(N, UU, VV);
  if (NEIG > 0 && GEP) copy(N, BU, BV);

finish : {
  if (NEIG < NWANT) {
    S_.rinit = std::pow(RINITM, 1.0 / (NEIG + 1));
    if (NEIG > 0) {
      long jj = std::min<long>(NEIG, NWANT - NEIG);
      copy(N * jj, N * (NWANT - jj) + XX, XX);
      for (long i = 0; i < jj; ++i) { EIGS[i] = EIGS[NWANT - jj + i]; RES[i] = RES[NWANT - jj + i]; }
      copy(N, VV, N * NEIG + XX);
      if (GEP) {
        copy(N * jj, N * (NWANT - jj) + BX, BX);
        copy(N, BV, N * NEIG + BX);
      }
      EIGS[NEIG] = THETA;
      RES[NEIG] = NREIG;
      THETA2 = THETA;
    } else {
      copy(N, UU, XX);
      if (GEP) copy(N, BU, BX);
      EIGS[0] = THETA;
      RES[0] = NREIG;
      GAP = 0;
      sync();
      return;
    }
  } else {
    S_.rinit = std::pow(RINITM, 1.0 / NEIG);
  }
  sortev_dev(N, NEIG, XX, BX, EIGS, RES, GEP ? -4 : 4, 0.0);
  long ITARG = 0;
  if (ISERCH >= 2) {
    for (ITARG = 1; ITARG <= NEIG; ++ITARG)
      if (EIGS[ITARG - 1] > SIGMA) break;
  }
  if (ISERCH == 2)
    GAP = std::fabs(THETA2 - SIGMA) - std::max(std::fabs(EIGS[NEIG - 1] - SIGMA), std::fabs(EIGS[0] - SIGMA));
  else GAP = THETA2 - EIGS[NEIG - 1];
  double GG = (ISERCH == 2) ? EIGS[0] + EIGS[NEIG - 1] - 2 * SIGMA : RINF;
  long II, JJ;
  if (GG > 0) { II = 1; JJ = NEIG - 1; }
  else { II = 2; JJ = NEIG; }
  if (NEIG == 1) { II = 0; JJ = 0; }
  auto E = [&](long i) -> double& { return EIGS[i - 1]; };
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
      copy(N * Jc, N * (I - 1) + XX, VV);
      for (long ij = 0; ij < Jc; ++ij) {
        matvec(3, VV + ij * N, WW + ij * N, -1);
        ITER++;
      }
      for (long c = 0; c < Jc; ++c) {
        gemvc(N, (int)c + 1, VV, N, WW + c * N, t1.data());
        gemvc(N, (int)c + 1, WW, N, VV + c * N, t2.data());
        for (long r = 0; r <= c; ++r) X[MM + r + c * MOD] = 0.5 * (t1[r] + t2[r]);
      }
      int inf2 = 0;
      solprojep(Jc, X + MM, X + NP, MOD, SCLR1, SCLR2, Wr, 3, inf2, GEP);
      if (inf2 == 0) {
        std::vector<T> q(Jc * Jc);
        for (long c = 0; c < Jc; ++c)
          for (long r = 0; r < Jc; ++r) q[r + c * Jc] = todev(X[MM + r + c * MOD]);
        auto blk = [&](long src, long dst) {
          k::rmult<T>(N, (int)Jc, (int)Jc, D(src), N, q.data(), W->dtmp, S());
          CK(cudaMemcpyAsync(D(dst), W->dtmp, sizeof(T) * N * Jc, cudaMemcpyDeviceToDevice, S()));
        };
        blk(VV, N * (I - 1) + XX);
        blk(WW, VV);
        if (GEP) {
          copy(N * Jc, N * (I - 1) + BX, BV);
          blk(BV, N * (I - 1) + BX);
        }
        double NRC = 0;
        GL -= E(I);
        GR += E(I + Jc - 1);
        for (long ij = 1; ij <= Jc; ++ij) {
          double th = hre(X[NP + ij - 1]);
          E(I + ij - 1) = th;
          axpy(N, H(-th), N * (I + ij - 2) + BX, VV + N * (ij - 1));
          double nr = nrm2(N, VV + N * (ij - 1));
          if (GEP) nr /= nrm2(N, N * (I + ij - 2) + BX);
          Rr(I + ij - 1) = nr;
          NRC += nr * nr;
        }
        for (long ij = I; ij <= I + Jc - 1; ++ij)
          if (ij == ITARG) ITARG--;
        I += Jc;
        continue;
      }
    }
    matvec(3, N * (I - 1), VV, -1);
    ITER++;
    {
      double th = hre(dot(N, N * (I - 1) + XX, VV));
      axpy(N, H(-th), N * (I - 1) + BX, VV);
      double nr = nrm2(N, VV);
      if (GEP) nr /= nrm2(N, N * (I - 1) + BX);
      E(I) = th;
      Rr(I) = nr;
      if (I == ITARG) ITARG--;
    }
    I++;
  }
  sync();
}
}

template struct DevJd<double>;
template struct DevJd<zc>;

}  // namespace jdg
