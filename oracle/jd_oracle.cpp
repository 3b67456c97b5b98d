#include <cstdlib>
// Test infrastructure only: the CPU oracle of the JADAMILU drop-in.
//
// Restates, on the CPU and in plain loops, the reference's driver layer:
//   PJDRVCOM   src/jd/JDaux.F:5-544    (init, adaptive re-factorisation, dispatch)
//   PJDINIT    src/jd/JDaux.F:549-1325 (shift choice, factor, retries, SPD conversion)
//   MATVECA    src/jd/JDaux.F:3397-3418 (upper-stored Hermitian SpMV)
//   DGLPRECSETUP/DGLPRECSOL src/jd/dglprecsetup.c:11-82, dglprecsol.c:8-26
//   SYMILUPACKSAVEDIAG src/ilupack/symamgsavediag.c (Gershgorin shift)
//   dsymamgsol / sdsymamgsol src/ilupack/symilupacksol.c:60-128,
//     singlesymilupacksol.c:69-144 (preconditioner application; the
//     ICNTL(5)=1 variant demotes the right-hand side, solves in single
//     precision and promotes the result)
// around the JD core of jd_core.hpp.  The multilevel factor itself is the
// project's host factorisation (jadamilu_gb300/csrc/ildlc.hpp); the oracle
// applies it with sequential triangular solves.
//
// Pinned by the reference's own results (the user guide's sample outputs,
// tests/golden/userguide_kats.json), by eigenvalues of solvers that share no
// code with it (ARPACK Lanczos and shift-and-invert fixtures under
// tests/golden/), and its factor application by scipy triangular solves
// (tests/test_factor.py).
//
// Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// and reference arm only.  The GPU library never links or calls it.
#include <chrono>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "../jadamilu_gb300/csrc/ildlc.hpp"
#include "../jadamilu_gb300/csrc/tail_inverse.hpp"
#include "../jadamilu_gb300/csrc/block_plan.hpp"
#include "jd_core.hpp"

namespace orc {

// ordering weight of the triangular-solve depth (same default as the GPU library)
static double g_depth_weight = 64.0;
static double g_drop_schur = -1.0;  // IldlcParams::droptol_schur (negative: its default rule)
static int g_matching = 0;          // IldlcParams::matching
// factor form for matrices of at least g_coupled_min_n rows (the library's
// defaults: one global L, Schur-contribution drop rule, look-ahead pivot
// deferral, exact last level once a level's matrix is a third full); smaller
// ones keep IldlcParams' own
static int g_drop_rule = 1;         // IldlcParams::drop_rule
static int g_coupling = 0;          // IldlcParams::coupling
static double g_last_droptol = 0;   // IldlcParams::last_droptol
static double g_last_fill = 1.0 / 3.0;  // IldlcParams::last_fill
static int g_coupled_min_n = 4096;
static int g_large_form_isearch = 2;  // solves take that form with ISEARCH at least this
static int g_lookahead = 1;         // IldlcParams::lookahead
static void factor_form(jdg::IldlcParams& p, int n, int isearch = 2) {
  if (n < g_coupled_min_n || isearch < g_large_form_isearch) return;
  p.lookahead = g_lookahead;
  p.coupling = g_coupling;
  p.drop_rule = g_drop_rule;
  p.last_droptol = g_last_droptol;
  p.last_fill = g_last_fill;
}
static int g_dense_min_rows = -1;   // IldlcParams::dense_min_rows (negative: its default)

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// MATVECA: y = A x, A Hermitian given by one triangle, diagonal first per row.
template <class T> void matveca(int n, const int* ia, const int* ja, const T* a, const T* x, T* y) {
  for (int i = 0; i < n; ++i) y[i] = T(0);
  for (int i = 0; i < n; ++i) {
    int k = ia[i] - 1;
    y[i] += a[k] * x[i];
    for (k = ia[i]; k < ia[i + 1] - 1; ++k) {
      int j = ja[k] - 1;
      y[i] += a[k] * x[j];
      y[j] += cj(a[k]) * x[i];
    }
  }
}

// Solve with one level's block B_l = L_l D_l L_l^H (|D_l| when spd) in place
// on v[a, e): the level's rows of L reference only columns in [a, e).
template <class T, class S>
void level_bsolve(const jdg::IldlcFactor<T>& F, bool spd, int a, int e, std::vector<S>& v) {
  for (int p = a; p < e; ++p) {
    S s = v[p];
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) s -= S(F.lx[q]) * v[F.li[q]];
    v[p] = s;
  }
  const std::vector<T>& di = spd ? F.ainv : F.dinv;
  const std::vector<T>& dof = spd ? F.aoff : F.doff;
  for (int p = a; p < e; ++p) {
    if (F.blk[p] == 1) {
      v[p] = S(di[p]) * v[p];
    } else if (F.blk[p] == 2) {
      S a0 = v[p], a1 = v[p + 1];
      S o = S(dof[p]);
      v[p] = S(di[p]) * a0 + o * a1;
      v[p + 1] = cj(o) * a0 + S(di[p + 1]) * a1;
      ++p;
    }
  }
  for (int p = e - 1; p >= a; --p) {
    S w = v[p];
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) v[F.li[q]] -= cj(S(F.lx[q])) * w;
  }
}

// Multilevel application with the coupling blocks (the block solve of
// symAMGsol.c:173-330): per level l, with the level's rows B and the later
// rows C,
//   forward:  y_B = B^{-1} b_B,  b_C -= F^H y_B   (then the next level on C),
//   backward: x_B = y_B - B^{-1} (F x_C).
// With spd every B^{-1} uses |D|, which keeps the operator Hermitian positive
// definite: it is P^H diag(|B|^{-1}, |S|^{-1}) P with P = [I 0; -F^H |B|^{-1} I].
template <class T, class S>
void ildl_apply_coupled(const jdg::IldlcFactor<T>& F, bool spd, const T* b, T* x, std::vector<S>& y) {
  const int n = F.n;
  const int nlev = (int)F.level_start.size() - 1;
  y.resize(n);
  std::vector<S> yb(n), t(n);
  for (int p = 0; p < n; ++p) y[p] = S(b[F.perm[p]]);
  for (int l = 0; l < nlev; ++l) {
    const int a = F.level_start[l], e = F.level_start[l + 1];
    level_bsolve(F, spd, a, e, y);
    if (l == nlev - 1) break;
    for (int p = a; p < e; ++p) {
      yb[p] = y[p];
      for (int64_t q = F.fp[p]; q < F.fp[p + 1]; ++q) y[F.fi[q]] -= cj(S(F.fx[q])) * y[p];
    }
  }
  for (int l = nlev - 2; l >= 0; --l) {
    const int a = F.level_start[l], e = F.level_start[l + 1];
    for (int p = a; p < e; ++p) {
      S s = S(0);
      for (int64_t q = F.fp[p]; q < F.fp[p + 1]; ++q) s += S(F.fx[q]) * y[F.fi[q]];
      t[p] = s;
    }
    level_bsolve(F, spd, a, e, t);
    for (int p = a; p < e; ++p) y[p] = yb[p] - t[p];
  }
  for (int p = 0; p < n; ++p) x[F.perm[p]] = T(y[p]);
}

// Application of the factor: x = P (L D L^H)^{-1} P^T b, with |D| when spd.
template <class T, class S>
void ildl_apply(const jdg::IldlcFactor<T>& F, bool spd, const T* b, T* x, std::vector<S>& y) {
  if (F.coupling == 1) {
    ildl_apply_coupled(F, spd, b, x, y);
    return;
  }
  const int n = F.n;
  y.resize(n);
  for (int p = 0; p < n; ++p) y[p] = S(b[F.perm[p]]);
  for (int p = 0; p < n; ++p) {
    S s = y[p];
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) s -= S(F.lx[q]) * y[F.li[q]];
    y[p] = s;
  }
  const std::vector<T>& di = spd ? F.ainv : F.dinv;
  const std::vector<T>& dof = spd ? F.aoff : F.doff;
  for (int p = 0; p < n; ++p) {
    if (F.blk[p] == 1) {
      y[p] = S(di[p]) * y[p];
    } else if (F.blk[p] == 2) {
      S a0 = y[p], a1 = y[p + 1];
      S o = S(dof[p]);
      y[p] = S(di[p]) * a0 + o * a1;
      y[p + 1] = cj(o) * a0 + S(di[p + 1]) * a1;
      ++p;
    }
  }
  for (int p = n - 1; p >= 0; --p) {
    S v = y[p];
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) y[F.li[q]] -= cj(S(F.lx[q])) * v;
  }
  for (int p = 0; p < n; ++p) x[F.perm[p]] = T(y[p]);
}

template <class T> struct LowT;
template <> struct LowT<double> { using type = float; };
template <> struct LowT<cplx> { using type = std::complex<float>; };

// SYMILUPACKSAVEDIAG: Gershgorin-type lower bound used as the default shift.
template <class T> double savediag_shift(int n, const int* ia, const int* ja, const T* a) {
  std::vector<double> disc(n, 0.0), dg(n, 0.0);
  int ki = 0;
  double ti = 0;
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j) {
      int k = ja[j - 1] - 1;
      if (k == i) {
        dg[i] = re(a[j - 1]);
        if (i == 0) ti = re(a[j - 1]);
        else {
          if (re(a[j - 1]) < ti) ti = re(a[j - 1]);
          ki = i;
        }
      } else {
        double v = ab(a[j - 1]);
        disc[i] += v;
        disc[k] += v;
      }
    }
  double val = ti - disc[ki];
  for (int i = 0; i < n; ++i) {
    double tmp = dg[i] - disc[i];
    if (tmp < val && dg[i] - ti < disc[ki]) val = tmp;
  }
  return val;
}

// SYMILUPACKSAVEDIAGGEP (symamgsavediaggep.c): the same bound for the pencil,
// after a symmetric diagonal scaling from B's row sums.
template <class T>
double savediag_shift_gep(int n, const int* ia, const int* ja, const T* a, const int* ib, const int* jb, const T* b) {
  std::vector<double> disc(n, 0.0), dg(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = ib[i]; j < ib[i + 1]; ++j)
      if (jb[j - 1] - 1 == i) dg[i] = re(b[j - 1]);
  for (int i = 0; i < n; ++i)
    for (int j = ib[i]; j < ib[i + 1]; ++j) {
      int k = jb[j - 1] - 1;
      if (k != i) {
        double val = std::sqrt(dg[i] / dg[k]);
        dg[i] += ab(b[j - 1]) * val;
        dg[k] += ab(b[j - 1]) / val;
      }
    }
  for (int i = 0; i < n; ++i) dg[i] = 1 / std::sqrt(dg[i]);
  int ki = 0;
  double ti = 0;
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j) {
      int k = ja[j - 1] - 1;
      if (k == i) {
        double val = dg[i] * re(a[j - 1]) * dg[k];
        if (i == 0) ti = val;
        else if (val < ti) { ti = val; ki = i; }
      } else {
        double val = dg[i] * ab(a[j - 1]) * dg[k];
        disc[i] += val;
        disc[k] += val;
      }
    }
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j)
      if (ja[j - 1] - 1 == i) dg[i] = dg[i] * re(a[j - 1]) * dg[i];
  double val = ti - disc[ki];
  for (int i = 0; i < n; ++i) {
    double tmp = dg[i] - disc[i];
    if (tmp < val && dg[i] - ti < disc[ki]) val = tmp;
  }
  return val;
}

struct PrecondFailure {};

// COMMON /PJDINITPJD/ and /ILUPACKMEM/ of the reference, one per precision.
template <class T> struct Global {
  double timefact = -1, shift0 = 0, droptol0 = 0, diagmin = 0, shiftmax = 0, memrequested = 0, memused = 0,
         condest0 = 5;
  const double slightlyless = 0.8, toldiv = 2.0;
  int factdgl = 0, factspd = 0, prvdr = 0;
  bool reenterfirsttime = false, flagsingle = false;
  jdg::IldlcFactor<T> F;
  std::vector<double> diag;  // diagonal preconditioner 1/(a_ii - shift)
  JdShared sh;
  int nfactor = 0;  // factorisations performed (diagnostic)
  void cleanup1() {
    factdgl = 0;
    F = jdg::IldlcFactor<T>();
    diag.clear();
  }
};
template <class T> Global<T>& G() {
  static Global<T> g;
  return g;
}

// DGLPRECSETUP (a holds the n diagonal entries)
template <class T> void dglprecsetup(Global<T>& g, const T* a, int n, int isearch, double shift, double& shift0) {
  g.diag.assign(n, 0.0);
  double dmin = re(a[0]), ta = dmin;
  for (int i = 1; i < n; ++i) {
    dmin = std::min(dmin, re(a[i]));
    ta = std::max(ta, re(a[i]));
  }
  g.diagmin = dmin;
  double ati = std::fabs(dmin), ata = std::min(std::fabs(ta), ati);
  double del = std::max(ta - dmin, ata);
  if (isearch <= 1) {
    shift0 = dmin - del / n;
    g.factspd = -1;
    if (isearch == 1 && shift < dmin) {
      shift0 = shift;
      g.factspd = 0;
    }
    for (int i = 0; i < n; ++i) g.diag[i] = 1.0 / (re(a[i]) - shift0);
  } else {
    g.factspd = 0;
    del = 1.0 / del;
    for (int i = 0; i < n; ++i) {
      double t = re(a[i]) - shift0;
      t = (t > 0) ? std::max(t, del) : std::min(t, -del);
      g.diag[i] = 1.0 / t;
    }
  }
  g.factdgl = 1;
}

// swap the diagonal entry to the front of each row (JDaux.F:215-229, 1010-1023)
template <class T> void diag_first(int n, int* ia, int* ja, T* a) {
  for (int i = 0; i < n; ++i)
    for (int j = ia[i] - 1; j < ia[i + 1] - 1; ++j)
      if (ja[j] - 1 == i) {
        int l = ia[i] - 1;
        std::swap(ja[j], ja[l]);
        std::swap(a[j], a[l]);
      }
}

// PJDINIT.  Returns ierr (0 ok).
template <class T>
int pjdinit(Global<T>& g, int n, T* a, int* ja, int* ia, const T* b, const int* jb, const int* ib, double sigma,
            int isearch, double& SHIFT, double& DROPTOL, double& MEM, const int* icntl, bool gep) {
  if (g.factdgl != 0) g.cleanup1();
  if (ja[0] < 0) {
    if (isearch >= 2) g.shift0 = sigma;
    double s0 = g.shift0;
    dglprecsetup(g, a, n, isearch, SHIFT, s0);
    g.shift0 = s0;
    return 0;
  }
  if (DROPTOL < 0) DROPTOL = 1e-2;
  double condest = (g.timefact > 0) ? g.condest0 : (icntl[3] <= 0 ? 5.0 : (double)icntl[3]);
  if (MEM <= 0) MEM = 10.0;
  int newsh = 0;
  for (;;) {
    double tic = now_s();
    g.diagmin = 0;
    for (int i = 0; i < n; ++i) {
      double val = 0;
      for (int j = ia[i] - 1; j < ia[i + 1] - 1; ++j)
        if (ja[j] - 1 == i) val = re(a[j]);
      g.diagmin = (i == 0) ? val : std::min(val, g.diagmin);
    }
    g.shift0 = savediag_shift(n, ia, ja, a);
    if (gep) g.shift0 = savediag_shift_gep(n, ia, ja, a, ib, jb, b);
    if (isearch >= 2) g.shift0 = sigma;
    int ggsh = 0;
    if (isearch == 1 && SHIFT < g.diagmin) g.shift0 = SHIFT;
    else ggsh = 1;
    if (isearch <= 0 && newsh == 1) g.shift0 = SHIFT;
    if (newsh != 1 && g.timefact <= 0) g.shiftmax = g.diagmin;
    g.memrequested = MEM;
    const int recompilu = (icntl[1] == 0 || icntl[1] == -2) ? 1 : -1;
    const double nposeig = (icntl[2] <= 0) ? 0.01 : 0.0;
    jdg::IldlcParams prm;
    prm.depth_weight = g_depth_weight;
    prm.droptol_schur = g_drop_schur;
    prm.matching = g_matching;
    factor_form(prm, n, isearch);
    prm.verbose = std::getenv("JDG_FACTOR_VERBOSE") ? 1 : 0;
    if (g_dense_min_rows >= 0) prm.dense_min_rows = g_dense_min_rows;
    prm.droptol = DROPTOL;
    prm.condest = condest;
    prm.mem = MEM;
    int ierr = jdg::ildlc_factor<T>(n, ia, ja, a, g.shift0, gep ? ib : nullptr, gep ? jb : nullptr,
                                    gep ? b : nullptr, prm, g.F);
    g.nfactor++;
    g.memused = (ierr == 0) ? g.F.fill() + 0.05 : MEM;
    diag_first(n, ia, ja, a);
    if (ierr == -3 || ierr == -2) {
      if (!(recompilu == -1 || g.prvdr == -1)) {
        g.prvdr = 1;
        DROPTOL = DROPTOL * 2 * g.toldiv;
        g.cleanup1();
        continue;
      }
    } else if (ierr == -5 || ierr == -6 || ierr > 0) {
      if (!(recompilu == -1 || g.prvdr == 1) && g.memused < g.slightlyless * g.memrequested) {
        if (g.memused < (3 * g.slightlyless - 2) * g.memrequested) DROPTOL /= 4 * g.toldiv;
        else if (g.memused < (2 * g.slightlyless - 1) * g.memrequested) DROPTOL /= 2 * g.toldiv;
        else DROPTOL /= g.toldiv;
        DROPTOL = std::max(DROPTOL, 1.01 * std::sqrt(DBL_EPSILON * 0.5));
        g.prvdr = -1;
        g.cleanup1();
        continue;
      }
    }
    if (ierr != 0) {
      g.cleanup1();
      return ierr;
    }
    double totaltime = now_s() - tic;
    g.factspd = 0;
    if (isearch <= 1) {
      g.factspd = g.F.nneg;
      if (g.factspd > 0) {
        if (!(recompilu == -1 || g.factspd <= n * nposeig)) {
          g.shiftmax = std::min(g.shift0, g.shiftmax);
          SHIFT = 2 * SHIFT - g.diagmin;
          newsh = 1;
          g.prvdr = std::min(g.prvdr, 0);
          g.cleanup1();
          continue;
        }
      } else if (isearch <= 0 || newsh == 1 || ggsh == 1) {
        g.factspd = -1;
      }
    }
    g.timefact = std::max(totaltime, 1e-2);
    g.factdgl = -1;
    g.droptol0 = DROPTOL;
    g.condest0 = condest;
    return 0;
  }
}

template <class T> struct PjdCtx {
  Global<T>* g;
  int n;
  T *a, *b;
  int *ia, *ja, *ib, *jb;
  bool gep, single;
  // adaptive re-factorisation inputs
  int* neig;
  double* eigs;
  double* gap;
  int nw, isearch;
  const int* icntl;
  double sigma, tol;
  double *shift, *droptol, *mem;
  double tic = 0, rprev = 1;
  // user matvec (reverse-communication emulation); nullptr: MATVECA
  void (*user_mv)(void*, int, const T*, T*, T*) = nullptr;
  void* user_ctx = nullptr;
  std::vector<typename LowT<T>::type> ylo;
  std::vector<T> yhi;
};

template <class T> void pjd_matvec(void* c, int which, const T* x, T* y, T* by) {
  PjdCtx<T>& C = *(PjdCtx<T>*)c;
  if (C.user_mv) { C.user_mv(C.user_ctx, which, x, y, by); return; }
  if (which == 1 || which == 3) matveca(C.n, C.ia, C.ja, C.a, x, y);
  if ((which == 1 || which == 4) && C.gep) matveca(C.n, C.ib, C.jb, C.b, x, by);
}

template <class T> void pjd_precond(void* c, const T* rhs, T* sol) {
  PjdCtx<T>& C = *(PjdCtx<T>*)c;
  Global<T>& g = *C.g;
  JdShared& S = g.sh;
  const double EPSMACH = DBL_EPSILON * 0.5;
  const int* icntl = C.icntl;
  const int NEIG = *C.neig, NW = C.nw;
  double* EIGS = C.eigs;
  double& SHIFT = *C.shift;
  double& DROPTOL = *C.droptol;
  bool reinit = false;
  int factspd0 = 0;
  double toc = now_s();
  auto E = [&](int i) { return EIGS[i - 1]; };
  if (g.factdgl > 0 && !S.flagcg && C.isearch <= 1 && (icntl[1] == 0 || icntl[1] == -2) && icntl[0] != 2) {
    double tent;
    if (NEIG >= 1) { tent = E(NW); factspd0 = -1; }
    else {
      tent = S.shift1 - S.rcurr;
      factspd0 = -1;
      if (10 * S.rcurr >= g.diagmin - tent && S.shift1 > g.shift0) factspd0 = g.factspd;
    }
    if (g.diagmin > tent && factspd0 < 0 && 10 * std::fabs(g.shift0 - tent) >= (g.diagmin - g.shift0)) {
      SHIFT = tent;
      reinit = true;
    }
  }
  if (g.factdgl < 0 && !S.flagcg && (icntl[1] == 0 || icntl[1] == -2) && icntl[0] != 2 &&
      S.rcum - C.rprev <= 6 * std::log(S.rinit / C.tol)) {
    double tmsol = toc - C.tic, time0, time1;
    if (tmsol < 1e-1) tmsol = 0;
    if (S.rcum > C.rprev) {
      time1 = tmsol * std::log(S.rinit / C.tol) / (S.rcum - C.rprev);
      time0 = tmsol * std::log(S.rcurr / C.tol) / (S.rcum - C.rprev);
    } else {
      time1 = 4 * g.timefact;
      time0 = 6 * g.timefact;
    }
    if (2 * g.timefact < time1 && 4 * g.timefact < time0 + (NW - NEIG - 1) * time1) {
      if (g.factspd < 0) {
        double tent, delta;
        if (NEIG >= 1) {
          delta = (NEIG > 1) ? std::fabs(E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*C.gap, 0.0);
          tent = std::min(2 * g.shiftmax - E(NW), E(NW) - delta);
        } else {
          tent = std::min(2 * g.shiftmax - S.shift1, S.shift1 - S.rcurr - std::max(*C.gap, 0.0));
          if (2 * S.rcurr >= g.diagmin - tent) factspd0 = g.factspd;
        }
        if ((factspd0 == 0 || 4 * g.timefact < time0) && g.diagmin > tent && 2 * (tent - g.shift0) >= (g.diagmin - g.shift0)) {
          SHIFT = tent;
          C.rprev = S.rcum;
          reinit = true;
        }
      }
      if (factspd0 >= 0 && !reinit && g.memused < g.slightlyless * g.memrequested && g.prvdr <= 0 &&
          DROPTOL >= std::sqrt(EPSMACH)) {
        if (icntl[1] != -2) g.reenterfirsttime = false;
        double DT0 = DROPTOL;
        if (!g.reenterfirsttime) {
          if (g.memused < (3 * g.slightlyless - 2) * g.memrequested) DROPTOL /= 4 * g.toldiv;
          else if (g.memused < (2 * g.slightlyless - 1) * g.memrequested) DROPTOL /= 2 * g.toldiv;
          else DROPTOL /= g.toldiv;
          DROPTOL = std::max(DROPTOL, 1.01 * std::sqrt(EPSMACH));
        }
        C.rprev = S.rcum;
        reinit = true;
        if (DROPTOL == 1.01 * std::sqrt(EPSMACH) && DT0 == DROPTOL && !g.reenterfirsttime) reinit = false;
        g.reenterfirsttime = false;
        SHIFT = g.shift0;
        if (g.factspd > 0) {
          if (NEIG >= 1) {
            double delta = (NEIG > 1) ? (E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*C.gap, 0.0);
            SHIFT = std::min(std::min(2 * g.shift0 - E(NW), E(NW) - delta), g.shiftmax);
          } else if (g.shift0 > S.shift1) {
            SHIFT = std::min(S.shift1, g.shiftmax);
          }
        }
      } else if (g.factspd > 0) {
        if (NEIG >= 1) {
          if (g.shift0 > E(NW)) {
            double delta = (NEIG > 1) ? (E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*C.gap, 0.0);
            SHIFT = std::min(E(NW) - delta, g.shiftmax);
            C.rprev = S.rcum;
            reinit = true;
          }
        } else if (g.shift0 > S.shift1 && 2 * (g.shift0 - S.shift1) >= (g.diagmin - g.shift0)) {
          SHIFT = std::min(S.shift1, g.shiftmax);
          C.rprev = S.rcum;
          reinit = true;
        }
      }
    }
  }
  if (reinit) {
    int ierr = pjdinit(g, C.n, C.a, C.ja, C.ia, C.b, C.jb, C.ib, C.sigma, std::max(C.isearch, 1), SHIFT, DROPTOL,
                       *C.mem, icntl, C.gep);
    if (ierr != 0) {
      g.factdgl = 1;
      throw PrecondFailure();
    }
    double t = now_s();
    S.timeilu += std::max(t - toc, 0.0);
    C.tic = t;
    if (factspd0 < 0 && g.factspd <= 0) g.factspd = factspd0;
  }
  if (g.factdgl > 0) {
    for (int i = 0; i < C.n; ++i) sol[i] = T(g.diag[i]) * rhs[i];
  } else if (C.single) {
    ildl_apply(g.F, C.isearch <= 1, rhs, sol, C.ylo);
  } else {
    ildl_apply(g.F, C.isearch <= 1, rhs, sol, C.yhi);
  }
}

// PJDRVCOM with the matvec done by MATVECA (or a user callback) and the
// preconditioner by the factor or the diagonal.
template <class T>
void pjd(int n, T* a, int* ja, int* ia, T* b, int* jb, int* ib, double* EIGS, double* RES, T* X, long LX, int& NEIG,
         double SIGMA, int ISEARCH, int NINIT, int MADSPACE, int& ITER, double TOL, double& SHIFT, double& DROPTOL,
         double& MEM, int* ICNTL, int& INFO, double& GAP, bool GEP, void (*user_mv)(void*, int, const T*, T*, T*),
         void* user_ctx) {
  Global<T>& g = G<T>();
  JdShared& S = g.sh;
  g.flagsingle = ICNTL[4] != 0;
  int ierr = 0;
  double t0 = now_s();
  if ((ICNTL[1] != -1 && ICNTL[1] != -2) || g.factdgl == 0) {
    g.prvdr = 0;
    g.timefact = -1;
    g.cleanup1();
    ierr = pjdinit(g, n, a, ja, ia, b, jb, ib, SIGMA, ISEARCH, SHIFT, DROPTOL, MEM, ICNTL, GEP);
    g.reenterfirsttime = false;
  } else {
    g.prvdr = 0;
    g.reenterfirsttime = true;
    S.rinit = S.rcurr = S.rcum = 0;
    if (ja[0] < 0) {
      if (ISEARCH >= 2) g.shift0 = SIGMA;
    } else {
      for (int i = 0; i < n; ++i) {
        double val = 0;
        for (int j = ia[i] - 1; j < ia[i + 1] - 1; ++j)
          if (ja[j] - 1 == i) val = re(a[j]);
        g.diagmin = (i == 0) ? val : std::min(val, g.diagmin);
      }
      if (!GEP) g.shift0 = savediag_shift(n, ia, ja, a);
      if (ISEARCH >= 2) g.shift0 = SIGMA;
      if (ISEARCH == 1 && SHIFT < g.diagmin) g.shift0 = SHIFT;
      diag_first(n, ia, ja, a);
      S.timeilu = 0;
    }
  }
  if (ierr != 0) {
    INFO = -54321;
    return;
  }
  PjdCtx<T> C;
  C.g = &g;
  C.n = n;
  C.a = a; C.b = b; C.ia = ia; C.ja = ja; C.ib = ib; C.jb = jb;
  C.gep = GEP;
  C.single = g.flagsingle;
  C.neig = &NEIG;
  C.eigs = EIGS;
  C.gap = &GAP;
  C.nw = NEIG;
  C.isearch = ISEARCH;
  C.icntl = ICNTL;
  C.sigma = SIGMA;
  C.tol = TOL;
  C.shift = &SHIFT;
  C.droptol = &DROPTOL;
  C.mem = &MEM;
  C.tic = now_s();
  C.rprev = 1.0;
  C.user_mv = user_mv;
  C.user_ctx = user_ctx;
  (void)t0;
  JdCore<T> core;
  core.sh = &S;
  core.cb.matvec = pjd_matvec<T>;
  core.cb.precond = pjd_precond<T>;
  core.cb.ctx = &C;
  try {
    core.run(n, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, INFO, GAP, GEP);
  } catch (PrecondFailure&) {
    INFO = -54321;
    return;
  }
  // suggested SHIFT / DROPTOL for a restart (JDaux.F:482-535)
  SHIFT = g.shift0;
  if (g.factdgl >= 0) {
    SHIFT = EIGS[0];
  } else if (g.factspd != 0 || ISEARCH <= 0) {
    double delta = (NEIG > 1) ? (EIGS[NEIG - 1] - EIGS[0]) / (NEIG - 1) : std::max(GAP, 0.0);
    if (g.factspd > 0) {
      SHIFT = std::min(SHIFT, g.shiftmax);
      SHIFT = std::min(2 * SHIFT - EIGS[0], EIGS[0] - delta);
    } else {
      SHIFT = std::min(2 * g.shiftmax - EIGS[0], EIGS[0] - delta);
      if (g.shift0 < EIGS[0]) SHIFT = std::max(SHIFT, g.shift0);
    }
  }
}

}  // namespace orc

using orc::cplx;
extern "C" {

typedef void (*orc_dmv_t)(void*, int, const double*, double*, double*);
typedef void (*orc_dpc_t)(void*, const double*, double*);
typedef void (*orc_zmv_t)(void*, int, const cplx*, cplx*, cplx*);
typedef void (*orc_zpc_t)(void*, const cplx*, cplx*);

// DJDREVCOM / DJDREVCOM_GEP semantics with callbacks in place of IJOB returns.
void orc_djd(int n, double* eigs, double* res, double* x, long lx, int* neig, double sigma, int isearch, int ninit,
             int madspace, int* iter, double tol, int* info, double* gap, int gep, orc_dmv_t mv, orc_dpc_t pc,
             void* ctx) {
  static orc::JdShared sh;
  orc::JdCore<double> core;
  core.sh = &sh;
  core.cb = {mv, pc, ctx};
  core.run(n, eigs, res, x, lx, *neig, sigma, isearch, ninit, madspace, *iter, tol, *info, *gap, gep != 0);
}
void orc_zjd(int n, double* eigs, double* res, cplx* x, long lx, int* neig, double sigma, int isearch, int ninit,
             int madspace, int* iter, double tol, int* info, double* gap, int gep, orc_zmv_t mv, orc_zpc_t pc,
             void* ctx) {
  static orc::JdShared sh;
  orc::JdCore<cplx> core;
  core.sh = &sh;
  core.cb = {mv, pc, ctx};
  core.run(n, eigs, res, x, lx, *neig, sigma, isearch, ninit, madspace, *iter, tol, *info, *gap, gep != 0);
}

// DPJD / DPJD_GEP (user_mv == NULL) and DPJDREVCOM (user_mv given).
void orc_dpjd(int n, double* a, int* ja, int* ia, double* b, int* jb, int* ib, double* eigs, double* res, double* x,
              long lx, int* neig, double sigma, int isearch, int ninit, int madspace, int* iter, double tol,
              double* shift, double* droptol, double* mem, int* icntl, int* info, double* gap, int gep,
              orc_dmv_t user_mv, void* user_ctx) {
  orc::pjd<double>(n, a, ja, ia, b, jb, ib, eigs, res, x, lx, *neig, sigma, isearch, ninit, madspace, *iter, tol,
                   *shift, *droptol, *mem, icntl, *info, *gap, gep != 0, user_mv, user_ctx);
}
void orc_zpjd(int n, cplx* a, int* ja, int* ia, cplx* b, int* jb, int* ib, double* eigs, double* res, cplx* x,
              long lx, int* neig, double sigma, int isearch, int ninit, int madspace, int* iter, double tol,
              double* shift, double* droptol, double* mem, int* icntl, int* info, double* gap, int gep,
              orc_zmv_t user_mv, void* user_ctx) {
  orc::pjd<cplx>(n, a, ja, ia, b, jb, ib, eigs, res, x, lx, *neig, sigma, isearch, ninit, madspace, *iter, tol,
                 *shift, *droptol, *mem, icntl, *info, *gap, gep != 0, user_mv, user_ctx);
}
void orc_dpjdcleanup(void) { orc::G<double>().cleanup1(); }

// Install an externally computed factor (same data layout as the project's
// host factor) as the current preconditioner, for runs with ICNTL(2) = -1.
void orc_dimport_factor(int n, const int* perm, const long long* lp, const int* li, const double* lx,
                        const signed char* blk, const double* dinv, const double* doff, const double* ainv,
                        const double* aoff, double shift0) {
  auto& g = orc::G<double>();
  g.cleanup1();
  auto& F = g.F;
  F.n = n;
  F.perm.assign(perm, perm + n);
  F.lp.assign(lp, lp + n + 1);
  F.li.assign(li, li + lp[n]);
  F.lx.assign(lx, lx + lp[n]);
  F.blk.assign(blk, blk + n);
  F.dinv.assign(dinv, dinv + n);
  F.doff.assign(doff, doff + n);
  F.ainv.assign(ainv, ainv + n);
  F.aoff.assign(aoff, aoff + n);
  F.level_start = {0, n};
  F.nnz_a_upper = 1;
  g.factdgl = -1;
  g.shift0 = shift0;
  g.timefact = 1.0;
  g.factspd = 0;
  g.memused = g.memrequested = 1e30;
}
// the level structure and coupling blocks of an imported factor (after orc_dimport_factor)
void orc_dimport_levels(int coupling, int nlev, const int* level_start, const long long* fp, const int* fi,
                        const double* fx) {
  auto& F = orc::G<double>().F;
  F.level_start.assign(level_start, level_start + nlev + 1);
  F.coupling = coupling;
  if (coupling == 1) {
    F.fp.assign(fp, fp + F.n + 1);
    F.fi.assign(fi, fi + fp[F.n]);
    F.fx.assign(fx, fx + fp[F.n]);
  }
}
void orc_zpjdcleanup(void) { orc::G<cplx>().cleanup1(); }
int orc_nfactor_d(void) { return orc::G<double>().nfactor; }

// MATVECA on its own (kernel parity).
void orc_dmatveca(int n, const int* ia, const int* ja, const double* a, const double* x, double* y) {
  orc::matveca(n, ia, ja, a, x, y);
}
void orc_zmatveca(int n, const int* ia, const int* ja, const cplx* a, const cplx* x, cplx* y) {
  orc::matveca(n, ia, ja, a, x, y);
}

// Factor (the project's host code) + the oracle's application of it, on an
// opaque handle, for kernel-level parity of the GPU preconditioner.
struct OrcFactorD { jdg::IldlcFactor<double> F; };
void orc_set_depth_weight(double w) { orc::g_depth_weight = w; }
void orc_set_drop_schur(double v) { orc::g_drop_schur = v; }
void orc_set_matching(int v) { orc::g_matching = v; }
void orc_set_drop_rule(int v) { orc::g_drop_rule = v; }
void orc_set_coupling(int v) { orc::g_coupling = v; }
void orc_set_last_level(double droptol, double fill) {
  orc::g_last_droptol = droptol;
  orc::g_last_fill = fill;
}
void orc_set_coupled_min_n(int v) { orc::g_coupled_min_n = v; }
void orc_set_large_form_isearch(int v) { orc::g_large_form_isearch = v; }
void orc_set_lookahead(int v) { orc::g_lookahead = v; }
// The dense-block inverse tiles (project code under test): L is unit lower
// triangular of order m given by rows rp/ci/cv (strictly lower, local
// columns).  Writes nt*(nt+1)/2 tiles of 64x64 doubles each into tf and tb;
// returns nt.
int orc_tail_inverse(int m, const long* rp, const int* ci, const double* cv, int threads, double* tf, double* tb) {
  std::vector<int64_t> p(rp, rp + m + 1);
  std::vector<int> c(ci, ci + rp[m]);
  std::vector<double> v(cv, cv + rp[m]);
  std::vector<double> f, b;
  jdg::tail_inverse<double, double>(m, p, c, v, f, b, threads, [](double x) { return x; });
  std::copy(f.begin(), f.end(), tf);
  std::copy(b.begin(), b.end(), tb);
  return (m + jdg::kTile - 1) / jdg::kTile;
}
// The small dense solvers shared by the oracle and the GPU driver
// (csrc/small_dense.hpp), column-major J x J, for tests against LAPACK.
int orc_heev(int cplx, int J, void* A, double* w) {
  return cplx ? jdd::heev<std::complex<double>>(J, (std::complex<double>*)A, J, w) : jdd::heev<double>(J, (double*)A, J, w);
}
int orc_hegv(int cplx, int J, void* A, void* B, double* w) {
  return cplx ? jdd::hegv<std::complex<double>>(J, (std::complex<double>*)A, J, (std::complex<double>*)B, J, w)
              : jdd::hegv<double>(J, (double*)A, J, (double*)B, J, w);
}
int orc_posv(int cplx, int J, void* N, void* M) {
  return cplx ? jdd::posv_u<std::complex<double>>(J, (std::complex<double>*)N, J, (std::complex<double>*)M, J)
              : jdd::posv_u<double>(J, (double*)N, J, (double*)M, J);
}
int orc_geev(int J, const double* A, double* wr, double* V) { return jdd::geev_right<double>(J, A, J, wr, V, J); }
void orc_householder_q(int K, int J, const double* U, double* Q) {
  std::vector<double> q;
  jdd::householder_q<double>(K, J, U, K, q);
  std::copy(q.begin(), q.end(), Q);
}
// the dense-block plan of a forward level structure (project code under
// test): writes 3 ints per group {first level, end level, dense}; returns
// the number of groups
int orc_plan_blocks(int nfl, const int* fptr, const long* ent_f, const long* ent_b, int elem_bytes, int dense_max,
                    double min_saving, int* out) {
  std::vector<int> fp(fptr, fptr + nfl + 1);
  std::vector<int64_t> ef(ent_f, ent_f + nfl), eb(ent_b, ent_b + nfl);
  std::vector<jdg::BlockGroup> g = jdg::plan_dense_blocks(fp, ef, eb, (size_t)elem_bytes, dense_max, min_saving);
  for (size_t i = 0; i < g.size(); ++i) {
    out[3 * i] = g[i].a;
    out[3 * i + 1] = g[i].b;
    out[3 * i + 2] = g[i].dense ? 1 : 0;
  }
  return (int)g.size();
}
// cluster work items of a tile set: 4 ints per item
int orc_cluster_items(int nt, int lower, int per_row, int* out) {
  std::vector<int> it = jdg::make_cluster_items(nt, lower != 0, per_row);
  std::copy(it.begin(), it.end(), out);
  return (int)it.size() / 4;
}
// the factor's matching scale (project code under test) for a full symmetric
// 0-based CSR pattern; returns the number of matched rows
int orc_matching_scale(int n, const int* rp, const int* ci, const double* av, double* scale) {
  std::vector<std::vector<int>> cols(n);
  std::vector<std::vector<double>> mods(n);
  for (int i = 0; i < n; ++i)
    for (int q = rp[i]; q < rp[i + 1]; ++q)
      if (av[q] != 0) {
        cols[i].push_back(ci[q]);
        mods[i].push_back(std::fabs(av[q]));
      }
  int nm = 0;
  std::vector<double> s = jdg::matching_scale(n, cols, mods, &nm);
  for (int i = 0; i < n; ++i) scale[i] = s[i];
  return nm;
}
void orc_set_dense_min_rows(int v) { orc::g_dense_min_rows = v; }
static int g_threads = 0;
void orc_set_threads(int t) { g_threads = t; }
void* orc_dfactor(int n, const int* ia, const int* ja, const double* a, double shift, double droptol, double condest,
                  double mem, int* ierr) {
  auto* h = new OrcFactorD;
  jdg::IldlcParams p;
  p.depth_weight = orc::g_depth_weight;
  p.droptol_schur = orc::g_drop_schur;
  p.matching = orc::g_matching;
  orc::factor_form(p, n);
  p.verbose = std::getenv("JDG_FACTOR_VERBOSE") ? 1 : 0;
  if (orc::g_dense_min_rows >= 0) p.dense_min_rows = orc::g_dense_min_rows;
  p.threads = g_threads;
  p.droptol = droptol;
  p.condest = condest;
  p.mem = mem;
  *ierr = jdg::ildlc_factor<double>(n, ia, ja, a, shift, nullptr, nullptr, nullptr, p, h->F);
  return h;
}
void orc_dfactor_info(void* h, long* out) {
  auto& F = ((OrcFactorD*)h)->F;
  std::vector<int> fp, fr, bp, br;
  jdg::ildlc_levels(F, fp, fr, bp, br);
  out[0] = F.n;
  out[1] = (long)F.li.size();
  out[2] = F.nneg;
  out[3] = (long)F.level_start.size() - 1;
  out[4] = (long)fp.size() - 1;
  out[5] = (long)bp.size() - 1;
  long n2 = 0;
  for (int p = 0; p < F.n; ++p) n2 += F.blk[p] == 2;
  out[6] = n2;
  out[7] = (long)F.fi.size();
}
// per elimination step: forward level; level_start boundaries into ls (size nlevels+1)
void orc_dfactor_levels(void* h, int* flev, int* ls) {
  auto& F = ((OrcFactorD*)h)->F;
  for (int p = 0; p < F.n; ++p) {
    int m = 0;
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) m = std::max(m, flev[F.li[q]] + 1);
    flev[p] = m;
  }
  for (size_t i = 0; i < F.level_start.size(); ++i) ls[i] = F.level_start[i];
}
// The factor's forward and backward level schedules (project code under
// test) and its L in CSR: sizes first (out[0..3] = nfwd levels, nbwd levels,
// n, nnz(L)), then with non-null arrays the schedules and L's pattern.
void orc_dfactor_schedule(void* h, long* sizes, int* fptr, int* frows, int* bptr, int* brows, long* lp, int* li) {
  auto& F = ((OrcFactorD*)h)->F;
  std::vector<int> fp, fr, bp, br;
  jdg::ildlc_levels(F, fp, fr, bp, br);
  sizes[0] = (long)fp.size() - 1;
  sizes[1] = (long)bp.size() - 1;
  sizes[2] = F.n;
  sizes[3] = (long)F.li.size();
  if (!fptr) return;
  std::copy(fp.begin(), fp.end(), fptr);
  std::copy(fr.begin(), fr.end(), frows);
  std::copy(bp.begin(), bp.end(), bptr);
  std::copy(br.begin(), br.end(), brows);
  for (int p = 0; p <= F.n; ++p) lp[p] = (long)F.lp[p];
  std::copy(F.li.begin(), F.li.end(), li);
}
void orc_dfactor_apply(void* h, int spd, int single, const double* b, double* x) {
  auto& F = ((OrcFactorD*)h)->F;
  if (single) {
    std::vector<float> y;
    orc::ildl_apply(F, spd != 0, b, x, y);
  } else {
    std::vector<double> y;
    orc::ildl_apply(F, spd != 0, b, x, y);
  }
}
// The arrays of a single-L factor (test infrastructure: a test rebuilds P, L
// and D^{-1} with scipy and checks the application against triangular
// solves that share no code with this file).  Sizes from
// orc_dfactor_schedule: n and nnz(L).
void orc_dfactor_export(void* h, int* perm, long* lp, int* li, double* lx, signed char* blk, double* dinv,
                        double* doff) {
  auto& F = ((OrcFactorD*)h)->F;
  std::copy(F.perm.begin(), F.perm.end(), perm);
  for (int p = 0; p <= F.n; ++p) lp[p] = (long)F.lp[p];
  std::copy(F.li.begin(), F.li.end(), li);
  std::copy(F.lx.begin(), F.lx.end(), lx);
  std::copy(F.blk.begin(), F.blk.end(), blk);
  std::copy(F.dinv.begin(), F.dinv.end(), dinv);
  std::copy(F.doff.begin(), F.doff.end(), doff);
}
void orc_dfactor_free(void* h) { delete (OrcFactorD*)h; }

}  // extern "C"
