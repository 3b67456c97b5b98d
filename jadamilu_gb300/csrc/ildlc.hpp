// Multilevel incomplete LDL^H factorisation with inverse-based pivoting
// ("ILDLC"), host side.  This is the project's own preconditioner set-up; it
// plays the role of the reference's ILUPACK chain
//   symilupackfactor.c:66-221 -> symAMGsetup.c:121-1646 -> sympiluc.F:169
// (scaling, fill-reducing ordering, Crout ILDL with inverse-based dropping and
// pivot deferral, 1x1/2x2 pivots, Schur-complement levels, dense last level,
// SPD conversion of symspd.c:37-1065) without being a port of it:
//
//  * scaling is symmetric max-norm equilibration of the current level and is
//    used only in the decisions (pivot tests, dropping), so the stored factor
//    needs no row/column scaling vectors at apply time;
//  * the ordering is a dynamic minimum-degree order on the incomplete
//    (dropped) pattern, chosen pivot by pivot;
//  * a pivot k is deferred to the next level when the running estimate of
//    |e_k^T L^{-1}| exceeds `condest`, or when neither a 1x1 pivot nor a 2x2
//    pivot with its strongest neighbour keeps the new L entries below
//    `condest`; deferred rows form the Schur complement of the level;
//  * the last level accepts every pivot with Bunch-Kaufman 1x1/2x2 choice;
//  * entries of L are dropped when |l_ik| * |e_k^T L^{-1}| <= droptol
//    (inverse-based dropping), fill of the Schur complement below droptol/10.
//
// All levels are folded into one permuted unit-lower L and a block-diagonal D:
//   P^T (A - shift I) P  ~=  L D L^H,
// with the levels recorded as ranges of elimination steps.  The GPU applies
// the factor by level-scheduled sweeps over L (forward) and L^H (backward).
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "matching.hpp"

namespace jdg {

using cplx = std::complex<double>;
inline double fre(double x) { return x; }
inline double fre(cplx x) { return x.real(); }
inline double fcj(double x) { return x; }
inline cplx fcj(cplx x) { return std::conj(x); }
inline double fab(double x) { return std::fabs(x); }
inline double fab(cplx x) { return std::abs(x); }

struct IldlcParams {
  double droptol = 1e-3;   // inverse-based drop tolerance for L
  double droptol_schur = -1;  // fill threshold for the Schur complement (<0: droptol/10)
  double condest = 5.0;    // bound on |e_k^T L^{-1}| (and on scaled L entries)
  double mem = 20.0;       // max (nnz(L)+n)/nnz(A_upper); <=0: unlimited
  int max_levels = 12;     // levels before the last (Bunch-Kaufman) level
  int last_level_min = 64; // a deferred set this small becomes the last level
  double min_progress = 0.05;  // a level accepting fewer than this fraction ends the recursion
  double depth_weight = 64.0;  // ordering key = degree + depth_weight * (forward level of the row)
  int threads = 0;             // host threads for the row updates (0: hardware concurrency, at most 16)
  double dense_fill = 0.25;    // a level whose active rows are at least this full is eliminated densely
  int dense_min_rows = 8192;   //   if it has at least this many rows (smaller ones are quick sparse)
  double dense_max_bytes = 16e9;  //   and its dense copy fits in this many bytes
  int matching = 0;            // 1: first level's decisions use the maximum-product matching scale;
                               // 2: also pivot matched 2-cycles of that level as 2x2 blocks first
  int coupling = 0;            // 0: one global unit L; the rows of deferred nodes keep their entries
                               //    in the columns of earlier levels (L21 = E B^{-1}, dropped);
                               // 1: per level, the coupling block F of the level's matrix (as in
                               //    ILUPACK's multilevel form, symAMGsol.c:173-330): L holds only the
                               //    entries inside each level, and an application solves with B twice
  double last_droptol = -1;    // drop tolerance of the last level (<0: droptol; 0: the last level is
                               // factored without dropping, like ILUPACK's dense last level,
                               // symAMGsetup.c:450-560); its Schur fill threshold is a tenth of it
  double last_fill = 0;        // > 0: a later level whose matrix is at least this fraction full becomes
                               // the last level (ILUPACK switches at one third)
  int lookahead = 0;           // 1: also defer a pivot whose kept column would raise a neighbour's
                               //    inverse estimate above condest (ILUPACK's improved estimate,
                               //    sympiluc.F:1440-1510: the pivot is skipped, not its neighbours)
  int verbose = 0;             // 1: one line per level on stderr (rows, accepted, entries, seconds)
  int drop_rule = 0;           // 0: drop l_ik when |l_ik| |e_k^T L^{-1}| <= droptol;
                               // 1: drop l_ik when its largest rank-1 term in the Schur complement,
                               //    |l_ik| |d_k| max_m |l_mk| (scaled), is <= droptol / kmax, kmax the
                               //    largest inverse estimate accepted so far in the level (the rule of
                               //    ILUPACK's sympiluc.F:2187-2240 with IMPROVED_ESTIMATE)
};

template <class T> struct IldlcFactor {
  int n = 0;
  std::vector<int> perm;        // perm[p] = original row (0-based) eliminated at step p
  std::vector<int64_t> lp;      // CSR of the strictly lower unit L, rows in elimination order
  std::vector<int> li;          //   column indices (elimination order, < row)
  std::vector<T> lx;            //   values
  std::vector<signed char> blk; // 1: 1x1 pivot, 2: first of a 2x2 pivot, -2: second of it
  std::vector<T> dinv;          // D^{-1}: 1x1 -> 1/d; 2x2 at (p,p+1): diag entries at p and p+1
  std::vector<T> doff;          // 2x2 D^{-1} off-diagonal (row p, col p+1) stored at p; (p+1,p) = conj
  std::vector<T> ainv, aoff;    // |D|^{-1} in the same layout (SPD conversion)
  std::vector<int> level_start; // elimination steps where each level starts, plus n
  int nneg = 0;                 // negative eigenvalues of D (pivots converted by |D|)
  int64_t nnz_a_upper = 0;
  // coupling == 1: per level l, the block F_l = S_l(B_l, C_l) of the level's matrix S_l between the
  // pivots accepted in the level (rows, elimination steps) and the nodes deferred from it (columns,
  // elimination steps of later levels); L has no entries across levels.  The preconditioner is
  //   M_l = [B_l  F_l; F_l^H  S_{l+1} + F_l^H B_l^{-1} F_l],  B_l = L_l D_l L_l^H.
  int coupling = 0;
  std::vector<int64_t> fp;      // CSR rows of F over all elimination steps (empty rows outside B_l)
  std::vector<int> fi;
  std::vector<T> fx;
  double fill() const {
    return (double)(li.size() + fi.size() + (size_t)n) / (double)std::max<int64_t>(1, nnz_a_upper);
  }
};

namespace detail {

template <class T> struct Ent { int col; T val; };

template <class T> struct Trailing {
  int n;
  std::vector<std::vector<Ent<T>>> rows;  // off-diagonal entries of the active matrix (full, Hermitian)
  std::vector<T> diag;
};

// bucket queue of nodes keyed by degree
struct DegQueue {
  std::vector<int> head, tail, next, prev, key;
  std::vector<char> in;
  int minkey = 0, count = 0;
  void init(int n, int maxkey) {
    head.assign(maxkey + 2, -1);
    tail.assign(maxkey + 2, -1);
    next.assign(n, -1);
    prev.assign(n, -1);
    key.assign(n, 0);
    in.assign(n, 0);
    minkey = 0;
    count = 0;
  }
  void grow(int k) {
    if (k + 2 > (int)head.size()) {
      head.resize(k + 2, -1);
      tail.resize(k + 2, -1);
    }
  }
  void push(int i, int k) {  // FIFO within a bucket
    grow(k);
    key[i] = k;
    prev[i] = tail[k];
    next[i] = -1;
    if (tail[k] >= 0) next[tail[k]] = i;
    else head[k] = i;
    tail[k] = i;
    in[i] = 1;
    if (k < minkey) minkey = k;
    ++count;
  }
  void remove(int i) {
    if (!in[i]) return;
    int k = key[i];
    if (prev[i] >= 0) next[prev[i]] = next[i];
    else head[k] = next[i];
    if (next[i] >= 0) prev[next[i]] = prev[i];
    else tail[k] = prev[i];
    in[i] = 0;
    --count;
  }
  void update(int i, int k) {
    if (!in[i] || key[i] == k) return;
    remove(i);
    push(i, k);
  }
  int pop() {
    if (count == 0) return -1;
    while (minkey < (int)head.size() && head[minkey] < 0) ++minkey;
    int i = head[minkey];
    remove(i);
    return i;
  }
};

// Fork-join pool for the row updates of one pivot: run(count, f) calls
// f(tid, i) for i in [0, count) spread over the threads, the caller
// included, and returns when all are done.  Workers spin between jobs.
class RowPool {
 public:
  explicit RowPool(int nthreads) : nt_(std::max(1, nthreads)) {
    for (int t = 1; t < nt_; ++t) th_.emplace_back([this, t] { loop(t); });
  }
  ~RowPool() {
    stop_.store(true);
    gen_.fetch_add(1);
    for (auto& t : th_) t.join();
  }
  int size() const { return nt_; }
  template <class F> void run(int count, F&& f) {
    if (nt_ == 1 || count < 2 * nt_) {
      for (int i = 0; i < count; ++i) f(0, i);
      return;
    }
    job_ = [&f](int tid, int i) { f(tid, i); };
    count_ = count;
    next_.store(0);
    done_.store(0);
    gen_.fetch_add(1, std::memory_order_release);
    work(0);
    while (done_.load(std::memory_order_acquire) < nt_ - 1) {
    }
  }

 private:
  void work(int tid) {
    for (;;) {
      int i = next_.fetch_add(1);
      if (i >= count_) break;
      job_(tid, i);
    }
  }
  void loop(int tid) {
    long seen = 0;
    for (;;) {
      long g;
      while ((g = gen_.load(std::memory_order_acquire)) == seen) {
      }
      seen = g;
      if (stop_.load()) return;
      work(tid);
      done_.fetch_add(1, std::memory_order_release);
    }
  }
  int nt_;
  std::vector<std::thread> th_;
  std::atomic<long> gen_{0};
  std::atomic<int> next_{0}, done_{0};
  std::atomic<bool> stop_{false};
  int count_ = 0;
  std::function<void(int, int)> job_;
};

}  // namespace detail

// Factor A - shift*B (B = identity when b == nullptr).  Inputs are the upper
// triangles in 1-based CSR exactly as the JADAMILU drivers receive them.
// Returns 0, -1 (bad input), -3 (fill above params.mem), or a positive step
// number for an exactly zero pivot in the last level.
template <class T>
int ildlc_factor(int n, const int* ia, const int* ja, const T* a, double shift, const int* ib, const int* jb,
                 const T* b, const IldlcParams& prm, IldlcFactor<T>& F) {
  using namespace detail;
  if (n <= 0) return -1;
  Trailing<T> A;
  A.n = n;
  A.rows.assign(n, {});
  A.diag.assign(n, T(0));
  const int64_t nnzu = (int64_t)ia[n] - ia[0];
  std::vector<int> cnt(n, 0);
  for (int i = 0; i < n; ++i)
    for (int64_t p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
      int j = ja[p] - 1;
      if (j < 0 || j >= n) return -1;
      if (j != i) { cnt[i]++; cnt[j]++; }
    }
  for (int i = 0; i < n; ++i) A.rows[i].reserve(cnt[i] + 8);
  for (int i = 0; i < n; ++i)
    for (int64_t p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
      int j = ja[p] - 1;
      T v = a[p];
      if (j == i) { A.diag[i] += T(fre(v)); continue; }
      // (i,j) holds A(i,j); row j gets A(j,i) = conj
      A.rows[i].push_back({j, v});
      A.rows[j].push_back({i, fcj(v)});
    }
  // merge duplicates
  {
    std::vector<int> mark(n, -1);
    for (int i = 0; i < n; ++i) {
      auto& r = A.rows[i];
      size_t w = 0;
      for (size_t q = 0; q < r.size(); ++q) {
        int c = r[q].col;
        if (mark[c] >= 0 && mark[c] < (int)w && r[mark[c]].col == c) { r[mark[c]].val += r[q].val; continue; }
        mark[c] = (int)w;
        r[w++] = r[q];
      }
      r.resize(w);
      for (auto& e : r) mark[e.col] = -1;
    }
  }
  if (!b)
    for (int i = 0; i < n; ++i) A.diag[i] -= T(shift);
  if (b) {
    for (int i = 0; i < n; ++i)
      for (int64_t p = ib[i] - 1; p < ib[i + 1] - 1; ++p) {
        int j = jb[p] - 1;
        T v = b[p];
        if (j == i) { A.diag[i] -= T(shift * fre(v)); continue; }
        T sv = T(-shift) * v;
        auto upd = [&](int r, int c, T val) {
          for (auto& e : A.rows[r])
            if (e.col == c) { e.val += val; return; }
          A.rows[r].push_back({c, val});
        };
        upd(i, j, sv);
        upd(j, i, fcj(sv));
      }
  }

  const double dropS = prm.droptol_schur >= 0 ? prm.droptol_schur : prm.droptol * 0.1;
  // drop thresholds of the current level (the last level may keep more, see last_droptol)
  double lvl_droptol = prm.droptol, lvl_dropS = dropS;
  const double kappa = prm.condest;
  double kmax_lvl = 1.0;  // largest inverse estimate accepted in the current level (drop_rule 1)
  // drop_rule 1: threshold on the scaled |l| of a column whose scaled pivot
  // magnitude is dsc and whose largest scaled entry is lmx
  auto crule_thr = [&](double nu, double dsc, double lmx) {
    kmax_lvl = std::max(kmax_lvl, nu);
    const double c = dsc * lmx;
    return c > 0 ? lvl_droptol / (kmax_lvl * c) : 0.0;
  };
  F = IldlcFactor<T>();
  F.n = n;
  F.nnz_a_upper = nnzu;
  std::vector<int> pos(n, -1);          // elimination step of each original row
  std::vector<int> order;               // original index per step
  order.reserve(n);
  std::vector<signed char> blk(n, 0);
  std::vector<T> dinv(n, T(0)), doff(n, T(0));
  // L by columns while factoring: for step p, entries (original row i, value)
  std::vector<int64_t> colptr;
  colptr.reserve(n + 1);
  colptr.push_back(0);
  std::vector<int> crow;
  std::vector<T> cval;
  crow.reserve((size_t)nnzu * 3);
  cval.reserve((size_t)nnzu * 3);
  const int64_t memcap = prm.mem > 0 ? (int64_t)(prm.mem * (double)nnzu) : INT64_MAX;
  const bool fform = prm.coupling == 1;
  // coupling 1: entries stored by the finished levels (their L and F), the
  // column entries at the start of the current level, the level's matrix
  // S_l(i, j) (i < j, node ids) and the F entries (accepted row, deferred column)
  int64_t stored_done = 0, crow_lvl0 = 0;
  struct Trip { int r, c; T v; };
  std::vector<Trip> snap, fent;
  std::vector<int> node_level(n, 0);
  // within a level, the column entries of L include those of the deferred rows
  // (E B^{-1}, not stored with coupling 1): a guard against runaway fill
  auto over_mem = [&]() {
    if (!fform) return (int64_t)crow.size() + n > memcap;
    const int64_t cur = stored_done + ((int64_t)crow.size() - crow_lvl0) + (int64_t)fent.size();
    return memcap < INT64_MAX / 4 && cur + n > 3 * memcap;
  };

  std::vector<char> state(n, 0);  // 0 active candidate, 1 eliminated, 2 deferred
  std::vector<double> sc(n, 1.0), xi(n, 0.0);
  std::vector<cplx> xic(n, cplx(0));  // complex estimator accumulators
  std::vector<int> slot(n, -1);
  const int nthr = prm.threads > 0 ? prm.threads
                                   : (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
  RowPool pool(n >= 20000 ? nthr : 1);
  // Stamped column -> position maps of the 1x1 row updates, one per thread:
  // an entry is valid when its stamp is the current update's, so the map
  // needs no clearing pass between rows.
  struct PosStamp { uint32_t stamp; int pos; };
  std::vector<std::vector<PosStamp>> tpos(pool.size());
  for (auto& v : tpos) v.assign(n, PosStamp{0u, -1});
  std::vector<uint32_t> tstamp(pool.size(), 0u);
  std::vector<char> inkept(n, 0);
  std::vector<int> mate(n, -1);  // matched 2-cycle partner (first level, matching = 2)
  std::vector<int> nbr;
  std::vector<int> dlev(n, 0);  // forward level row i would get if eliminated now
  auto qkey = [&](int i) { return (int)A.rows[i].size() + (int)(prm.depth_weight * dlev[i]); };
  std::vector<int> level_nodes(n);
  for (int i = 0; i < n; ++i) level_nodes[i] = i;
  DegQueue Q;
  int level = 0;
  bool last = false;
  std::vector<int> kept;
  std::vector<T> lk, lj;  // L column values (unscaled) for the pivot(s)
  std::vector<T> tmpv;
  const bool is_cplx = !std::is_same<T, double>::value;

  auto remove_col = [&](int r, int c) {
    auto& row = A.rows[r];
    for (size_t q = 0; q < row.size(); ++q)
      if (row[q].col == c) { row[q] = row.back(); row.pop_back(); return; }
  };

  // Dense elimination of one level (its active rows nearly full): the same
  // pivot rules, dropping, estimator and ordering key (row count + depth
  // weight x forward level, dynamic) as the sparse loop below, on a dense
  // copy M of the level's active matrix (M[r*m + c] = A(nodes[r], nodes[c])).
  // An entry that is exactly zero counts as absent for the Schur-fill
  // dropping and for the row counts.  The rows of the deferred nodes are
  // written back as sparse rows.
  std::vector<int> dloc(n, -1);
  auto dense_level = [&](const std::vector<int>& nodes, bool last_lvl, std::vector<int>& deferred,
                         int& accepted) -> int {
    const int m = (int)nodes.size();
    for (int t = 0; t < m; ++t) dloc[nodes[t]] = t;
    std::vector<T> M((size_t)m * m, T(0));
    for (int t = 0; t < m; ++t) {
      const int i = nodes[t];
      M[(size_t)t * m + t] = A.diag[i];
      for (auto& e : A.rows[i]) M[(size_t)t * m + dloc[e.col]] = e.val;
      A.rows[i].clear();
      A.rows[i].shrink_to_fit();
    }
    std::vector<double> s(m);
    for (int t = 0; t < m; ++t) s[t] = sc[nodes[t]];
    std::vector<char> st(m, 0);  // 0 candidate, 1 eliminated, 2 deferred
    std::vector<int> cnt(m, 0);  // nonzeros of each row among the columns not eliminated
    for (int t = 0; t < m; ++t)
      for (int c = 0; c < m; ++c)
        if (c != t && M[(size_t)t * m + c] != T(0)) cnt[t]++;
    auto dkey = [&](int t) { return cnt[t] + (int)(prm.depth_weight * dlev[nodes[t]]); };
    DegQueue DQ;
    {
      int mk = 0;
      for (int t = 0; t < m; ++t) mk = std::max(mk, dkey(t));
      DQ.init(m, mk + 1);
      for (int t = 0; t < m; ++t) DQ.push(t, dkey(t));
    }
    // a column leaves the active matrix: the rows holding it lose one entry
    auto drop_column = [&](int p) {
      for (int r = 0; r < m; ++r)
        if (r != p && st[r] != 1 && M[(size_t)r * m + p] != T(0)) cnt[r]--;
    };
    std::vector<T> lf(m), lg(m);  // dense L columns (zero where dropped or eliminated)
    std::vector<int> kr;          // local rows with a kept entry
    auto nu_of = [&](int i) { return 1.0 + (is_cplx ? std::abs(xic[i]) : std::fabs(xi[i])); };
    auto at = [&](int r, int c) -> T& { return M[(size_t)r * m + c]; };
    // M(r, c) -= a_r * conj(b_c) (+ c_r * conj(d_c)) for rows and columns in
    // kr (the only columns with a nonzero L entry); fill drop
    auto update_rows = [&](const std::vector<T>& av, const std::vector<T>& bv, const std::vector<T>* cv,
                           const std::vector<T>* dv) {
      pool.run((int)kr.size(), [&](int, int q) {
        const int r = kr[q];
        const T ar = av[r], cr = cv ? (*cv)[r] : T(0);
        T* row = M.data() + (size_t)r * m;
        const double sr = s[r];
        for (int c : kr) {
          if (c == r) continue;
          T u = ar * fcj(bv[c]);
          if (cv) u += cr * fcj((*dv)[c]);
          if (u == T(0)) continue;
          if (row[c] != T(0)) {
            row[c] -= u;
          } else if (fab(u) * sr * s[c] > lvl_dropS) {
            row[c] = -u;
            cnt[r]++;
          }
        }
        T ud = ar * fcj(bv[r]);
        if (cv) ud += cr * fcj((*dv)[r]);
        row[r] -= T(fre(ud));
      });
    };
    while (DQ.count > 0) {
      int t = DQ.pop();
      if (st[t] != 0) continue;
      int k = nodes[t];
      double nuk = nu_of(k);
      if (!last_lvl && nuk > kappa) { st[t] = 2; state[k] = 2; deferred.push_back(k); continue; }
      T dk = at(t, t);
      const double skt = s[t];
      double dks = fab(dk) * skt * skt;
      double cmax = 0, amax = 0;
      int jb = -1;
      for (int r = 0; r < m; ++r) {
        if (r == t || st[r] == 1) continue;
        const double v = fab(at(t, r)) * skt * s[r];
        cmax = std::max(cmax, v);
        if (st[r] == 0 && v > amax) { amax = v; jb = r; }
      }
      int piv = 0;
      if (last_lvl) {
        const double alpha = 0.6404;
        if (dks > 0 && dks >= alpha * cmax) piv = 1;
        else if (jb < 0) piv = dks > 0 ? 1 : -1;
        else {
          double omj = 0;
          for (int r = 0; r < m; ++r)
            if (r != t && r != jb && st[r] != 1) omj = std::max(omj, fab(at(jb, r)) * s[jb] * s[r]);
          const double djs = fab(at(jb, jb)) * s[jb] * s[jb];
          if (dks * omj >= alpha * amax * amax) piv = 1;
          else if (djs >= alpha * omj && djs >= alpha * amax) piv = 3;
          else piv = 2;
        }
        if (piv == -1) return (int)order.size() + 1;
      } else {
        if (dks > 0 && cmax <= kappa * dks) piv = 1;
        else if (jb >= 0 && nu_of(nodes[jb]) <= kappa) piv = 2;
        else piv = 0;
      }
      if (piv == 0) { st[t] = 2; state[k] = 2; deferred.push_back(k); continue; }
      int tp = t;  // local pivot row
      if (piv == 3) {  // pivot on jb alone; t goes back to the queue
        DQ.push(t, dkey(t));
        DQ.remove(jb);
        tp = jb;
        piv = 1;
      }
      if (piv == 1) {
        const int kk = nodes[tp];
        const T d = at(tp, tp);
        const double nx = last_lvl ? 1.0 : nu_of(kk);
        const double sp = s[tp];
        const bool crule = prm.drop_rule == 1 && !last_lvl;
        double cthr = 0;
        if (crule) {
          double lmx = 0;
          for (int r = 0; r < m; ++r)
            if (r != tp && st[r] != 1 && at(r, tp) != T(0)) lmx = std::max(lmx, fab(at(r, tp) / d) * s[r] / sp);
          cthr = crule_thr(nx, fab(d) * sp * sp, lmx);
        }
        kr.clear();
        std::fill(lf.begin(), lf.end(), T(0));
        for (int r = 0; r < m; ++r) {
          if (r == tp || st[r] == 1) continue;
          const T a_rk = at(r, tp);
          if (a_rk == T(0)) continue;
          const T l = a_rk / d;
          if (crule ? fab(l) * s[r] / sp <= cthr : fab(l) * s[r] / sp * nx <= lvl_droptol) continue;
          lf[r] = l;
          kr.push_back(r);
        }
        if (!last_lvl) {
          if (is_cplx) {
            cplx x = (std::abs(xic[kk]) > 0) ? -xic[kk] / std::abs(xic[kk]) * (1 + std::abs(xic[kk])) : cplx(1);
            for (int r : kr) xic[nodes[r]] += cplx(lf[r] * T(s[r] / sp)) * x;
          } else {
            double x = (xi[kk] != 0) ? -(xi[kk] / std::fabs(xi[kk])) * (1 + std::fabs(xi[kk])) : 1.0;
            for (int r : kr) xi[nodes[r]] += fre(lf[r]) * (s[r] / sp) * x;
          }
        }
        for (int r : kr) lg[r] = lf[r] * d;
        drop_column(tp);
        st[tp] = 1;  // column tp leaves the update
        update_rows(lg, lf, nullptr, nullptr);
        for (int r : kr) {
          dlev[nodes[r]] = std::max(dlev[nodes[r]], dlev[kk] + 1);
          lg[r] = T(0);
        }
        pos[kk] = (int)order.size();
        order.push_back(kk);
        blk[pos[kk]] = 1;
        dinv[pos[kk]] = T(1) / d;
        for (int r : kr) { crow.push_back(nodes[r]); cval.push_back(lf[r]); }
        colptr.push_back((int64_t)crow.size());
        state[kk] = 1;
        accepted++;
      } else {
        const int j = nodes[jb];
        const T akj = at(t, jb), dkk = at(t, t), djj = at(jb, jb);
        const T det = dkk * djj - akj * fcj(akj);
        const double sj = s[jb];
        const double dets = fab(det) * skt * skt * sj * sj, offs = fab(akj) * skt * sj;
        const bool ok = dets > 1e-3 * offs * offs && fab(det) > 0;
        const T i00 = djj / det, i11 = dkk / det, i01 = -akj / det, i10 = fcj(i01);
        std::fill(lf.begin(), lf.end(), T(0));
        std::fill(lg.begin(), lg.end(), T(0));
        double lmax = 0;
        std::vector<int> nb;
        for (int r = 0; r < m; ++r) {
          if (r == t || r == jb || st[r] == 1) continue;
          const T aik = at(r, t), aij = at(r, jb);
          if (aik == T(0) && aij == T(0)) continue;
          lf[r] = aik * i00 + aij * i10;
          lg[r] = aik * i01 + aij * i11;
          lmax = std::max(lmax, std::max(fab(lf[r]) * s[r] / skt, fab(lg[r]) * s[r] / sj));
          nb.push_back(r);
        }
        if (!last_lvl && (!ok || lmax > kappa)) { st[t] = 2; state[k] = 2; deferred.push_back(k); continue; }
        if (last_lvl && !(fab(det) > 0)) return (int)order.size() + 1;
        const double nxk = last_lvl ? 1.0 : nu_of(k), nxj = last_lvl ? 1.0 : nu_of(j);
        const bool crule = prm.drop_rule == 1 && !last_lvl;
        double thk = 0, thj = 0;
        if (crule) {
          double mk = 0, mj = 0;
          for (int r : nb) {
            mk = std::max(mk, fab(lf[r]) * s[r] / skt);
            mj = std::max(mj, fab(lg[r]) * s[r] / sj);
          }
          const double bd = std::max({fab(dkk) * skt * skt, fab(djj) * sj * sj, fab(akj) * skt * sj});
          thk = crule_thr(nxk, bd, mk);
          thj = crule_thr(nxj, bd, mj);
        }
        kr.clear();
        for (int r : nb) {
          if (crule ? fab(lf[r]) * s[r] / skt <= thk : fab(lf[r]) * s[r] / skt * nxk <= lvl_droptol) lf[r] = T(0);
          if (crule ? fab(lg[r]) * s[r] / sj <= thj : fab(lg[r]) * s[r] / sj * nxj <= lvl_droptol) lg[r] = T(0);
          if (lf[r] != T(0) || lg[r] != T(0)) kr.push_back(r);
        }
        if (!last_lvl) {
          if (is_cplx) {
            cplx xk = (std::abs(xic[k]) > 0) ? -xic[k] / std::abs(xic[k]) * (1 + std::abs(xic[k])) : cplx(1);
            cplx xj = (std::abs(xic[j]) > 0) ? -xic[j] / std::abs(xic[j]) * (1 + std::abs(xic[j])) : cplx(1);
            for (int r : nb)
              xic[nodes[r]] += cplx(lf[r] * T(s[r] / skt)) * xk + cplx(lg[r] * T(s[r] / sj)) * xj;
          } else {
            double xk = (xi[k] != 0) ? -(xi[k] / std::fabs(xi[k])) * (1 + std::fabs(xi[k])) : 1.0;
            double xj = (xi[j] != 0) ? -(xi[j] / std::fabs(xi[j])) * (1 + std::fabs(xi[j])) : 1.0;
            for (int r : nb) xi[nodes[r]] += fre(lf[r]) * (s[r] / skt) * xk + fre(lg[r]) * (s[r] / sj) * xj;
          }
        }
        // update_il = l_ik t_l0 + l_ij t_l1 with t_l = D [conj(l_lk); conj(l_lj)]:
        // M(r, c) -= (l_rk dkk + l_rj conj(akj)) conj(l_ck) + (l_rk akj + l_rj djj) conj(l_cj)
        std::vector<T> ua(m, T(0)), ub(m, T(0));
        for (int r : kr) {
          ua[r] = lf[r] * dkk + lg[r] * fcj(akj);
          ub[r] = lf[r] * akj + lg[r] * djj;
        }
        drop_column(t);
        st[t] = 1;
        drop_column(jb);
        st[jb] = 1;
        DQ.remove(jb);
        update_rows(ua, lf, &ub, &lg);
        const int lv = std::max(dlev[k], dlev[j]) + 1;
        for (int r : kr) dlev[nodes[r]] = std::max(dlev[nodes[r]], lv);
        pos[k] = (int)order.size();
        order.push_back(k);
        pos[j] = (int)order.size();
        order.push_back(j);
        blk[pos[k]] = 2;
        blk[pos[j]] = -2;
        dinv[pos[k]] = i00;
        dinv[pos[j]] = i11;
        doff[pos[k]] = i01;
        for (int r : kr)
          if (lf[r] != T(0)) { crow.push_back(nodes[r]); cval.push_back(lf[r]); }
        colptr.push_back((int64_t)crow.size());
        for (int r : kr)
          if (lg[r] != T(0)) { crow.push_back(nodes[r]); cval.push_back(lg[r]); }
        colptr.push_back((int64_t)crow.size());
        state[k] = 1;
        state[j] = 1;
        accepted += 2;
      }
      if (over_mem()) return -3;
      for (int r : kr)
        if (st[r] == 0) DQ.update(r, dkey(r));
    }
    // deferred rows back to the sparse trailing matrix
    for (int t = 0; t < m; ++t) {
      if (st[t] != 2) continue;
      const int i = nodes[t];
      A.diag[i] = at(t, t);
      for (int c = 0; c < m; ++c)
        if (c != t && st[c] == 2 && at(t, c) != T(0)) A.rows[i].push_back({nodes[c], at(t, c)});
    }
    for (int t = 0; t < m; ++t) dloc[nodes[t]] = -1;
    return 0;
  };

  double t_level0 = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  while (!level_nodes.empty()) {
    const int nl = (int)level_nodes.size();
    if (level >= prm.max_levels || nl <= prm.last_level_min) last = true;
    F.level_start.push_back((int)order.size());
    if (level == 0 && prm.matching) {
      // first level: the symmetric scale of a maximum-product matching
      // (decisions only, like the equilibration below)
      std::vector<std::vector<int>> mc(n);
      std::vector<std::vector<double>> mm(n);
      for (int i = 0; i < n; ++i) {
        if (fab(A.diag[i]) > 0) {
          mc[i].push_back(i);
          mm[i].push_back(fab(A.diag[i]));
        }
        for (auto& e : A.rows[i])
          if (fab(e.val) > 0) {
            mc[i].push_back(e.col);
            mm[i].push_back(fab(e.val));
          }
      }
      std::vector<int> col_of;
      const std::vector<double> ms = matching_scale(n, mc, mm, nullptr, &col_of);
      for (int i = 0; i < n; ++i) sc[i] = ms[i];
      if (prm.matching >= 2)  // pairs: matched 2-cycles off the diagonal
        for (int i = 0; i < n; ++i) {
          const int j = col_of[i];
          mate[i] = (j >= 0 && j != i && col_of[j] == i) ? j : -1;
        }
    } else {
      // symmetric max-norm scaling of the current level (decisions only)
      for (int i : level_nodes) {
        double m = fab(A.diag[i]);
        for (auto& e : A.rows[i])
          if (state[e.col] != 1) m = std::max(m, fab(e.val));
        sc[i] = m > 0 ? 1.0 / std::sqrt(m) : 1.0;
      }
      for (int sweep = 0; sweep < 2; ++sweep)
        for (int i : level_nodes) {
          double m = fab(A.diag[i]) * sc[i] * sc[i];
          for (auto& e : A.rows[i]) m = std::max(m, fab(e.val) * sc[i] * sc[e.col]);
          if (m > 0) sc[i] /= std::sqrt(m);
        }
    }
    std::vector<int> deferred;
    int accepted_here = 0;
    kmax_lvl = 1.0;
    int64_t level_entries = 0;
    for (int i : level_nodes) {
      xi[i] = 0;
      xic[i] = 0;
      state[i] = 0;
      level_entries += (int64_t)A.rows[i].size();
      node_level[i] = level;
    }
    if (fform) {
      // the level's matrix before its elimination: F is its accepted x deferred block
      crow_lvl0 = (int64_t)crow.size();
      snap.clear();
      for (int i : level_nodes) {
        dlev[i] = 0;  // levels have no dependencies across them
        for (auto& e : A.rows[i])
          if (i < e.col) snap.push_back({i, e.col, e.val});
      }
    }
    if (!last && level > 0 && prm.last_fill > 0 &&
        (double)level_entries >= prm.last_fill * (double)nl * (double)(nl - 1))
      last = true;
    lvl_droptol = (last && prm.last_droptol >= 0) ? prm.last_droptol : prm.droptol;
    lvl_dropS = (last && prm.last_droptol >= 0) ? 0.1 * prm.last_droptol : dropS;
    const bool dense_lvl = nl >= prm.dense_min_rows &&
                           (double)level_entries >= prm.dense_fill * (double)nl * (double)(nl - 1) &&
                           (double)nl * (double)nl * sizeof(T) <= prm.dense_max_bytes;
    if (dense_lvl) {
      const int rc = dense_level(level_nodes, last, deferred, accepted_here);
      if (rc != 0) return rc;
    }
    int maxdeg = 0;
    if (!dense_lvl) {
      for (int i : level_nodes) maxdeg = std::max(maxdeg, (int)A.rows[i].size());
      Q.init(n, maxdeg + 1);
      for (int i : level_nodes) Q.push(i, qkey(i));
    }

    while (!dense_lvl && Q.count > 0) {
      int k = Q.pop();
      if (state[k] != 0) continue;
      const double sk = sc[k];
      auto nu_of = [&](int i) { return 1.0 + (is_cplx ? std::abs(xic[i]) : std::fabs(xi[i])); };
      double nuk = nu_of(k);
      if (!last && nuk > kappa) { state[k] = 2; deferred.push_back(k); continue; }
      T dk = A.diag[k];
      double dks = fab(dk) * sk * sk;
      // largest scaled entry in column k, and the strongest active neighbour
      double cmax = 0, amax = 0;
      int jbest = -1;
      for (auto& e : A.rows[k]) {
        double v = fab(e.val) * sk * sc[e.col];
        cmax = std::max(cmax, v);
        if (state[e.col] == 0 && v > amax) { amax = v; jbest = e.col; }
      }
      int piv = 0;  // 0 defer, 1 one-by-one at k, 2 two-by-two (k, j), 3 one-by-one at jbest
      if (last) {
        const double alpha = 0.6404;
        if (dks > 0 && dks >= alpha * cmax) piv = 1;
        else if (jbest < 0) piv = dks > 0 ? 1 : -1;
        else {
          double sj = sc[jbest], omj = 0;
          for (auto& e : A.rows[jbest])
            if (e.col != k) omj = std::max(omj, fab(e.val) * sj * sc[e.col]);
          double djs = fab(A.diag[jbest]) * sj * sj;
          if (dks * omj >= alpha * amax * amax) piv = 1;
          else if (djs >= alpha * omj && djs >= alpha * amax) piv = 3;
          else piv = 2;
        }
        if (piv == -1) {  // structurally and numerically zero row: singular
          return (int)order.size() + 1;
        }
      } else {
        const int mk = level == 0 ? mate[k] : -1;
        if (mk >= 0 && state[mk] == 0 && nu_of(mk) <= kappa) {
          jbest = mk;  // the matching's pair as a 2x2 pivot
          piv = 2;
        } else if (dks > 0 && cmax <= kappa * dks) piv = 1;
        else if (jbest >= 0 && nu_of(jbest) <= kappa) piv = 2;
        else piv = 0;
      }
      int jp = (piv == 2 || piv == 3) ? jbest : -1;
      if (piv == 3) {  // pivot on jbest alone; k stays in the queue
        Q.push(k, qkey(k));
        k = jp;
        Q.remove(k);
        jp = -1;
        piv = 1;
        nuk = nu_of(k);
        dk = A.diag[k];
      }
      const double skk = sc[k];
      if (piv == 1) {
        // 1x1 pivot at k
        T d = dk;
        double nx = last ? 1.0 : nuk;
        const bool crule = prm.drop_rule == 1 && !last;
        double cthr = 0;
        if (crule) {
          double lmx = 0;
          for (auto& e : A.rows[k])
            if (state[e.col] != 1) lmx = std::max(lmx, fab(fcj(e.val) / d) * sc[e.col] / skk);
          cthr = crule_thr(nx, fab(d) * skk * skk, lmx);
        }
        kept.clear();
        lk.clear();
        for (auto& e : A.rows[k]) {
          if (state[e.col] == 1) continue;
          T l = fcj(e.val) / d;  // L(i,k) = A(i,k)/d, A(i,k) = conj(A(k,i))
          double ls = fab(l) * sc[e.col] / skk;
          if (crule ? ls <= cthr : ls * nx <= lvl_droptol) continue;
          kept.push_back(e.col);
          lk.push_back(l);
        }
        // (the row of every neighbour loses column k below)
        if (!last && prm.lookahead) {
          bool over = false;
          if (is_cplx) {
            cplx x = (std::abs(xic[k]) > 0) ? -xic[k] / std::abs(xic[k]) * (1 + std::abs(xic[k])) : cplx(1);
            for (size_t q = 0; q < kept.size() && !over; ++q)
              over = std::abs(xic[kept[q]] + cplx(lk[q] * T(sc[kept[q]] / skk)) * x) > kappa;
          } else {
            double x = (xi[k] != 0) ? -(xi[k] / std::fabs(xi[k])) * (1 + std::fabs(xi[k])) : 1.0;
            for (size_t q = 0; q < kept.size() && !over; ++q)
              over = std::fabs(xi[kept[q]] + fre(lk[q]) * (sc[kept[q]] / skk) * x) > kappa;
          }
          if (over) {
            state[k] = 2;
            deferred.push_back(k);
            continue;
          }
        }
        if (!last) {
          // estimator: choose x_k to maximise growth
          if (is_cplx) {
            cplx x = (std::abs(xic[k]) > 0) ? -xic[k] / std::abs(xic[k]) * (1 + std::abs(xic[k])) : cplx(1);
            for (size_t q = 0; q < kept.size(); ++q) {
              int i = kept[q];
              double r = sc[i] / skk;
              xic[i] += cplx(lk[q] * T(r)) * x;
            }
          } else {
            double x = (xi[k] != 0) ? -(xi[k] / std::fabs(xi[k])) * (1 + std::fabs(xi[k])) : 1.0;
            for (size_t q = 0; q < kept.size(); ++q) {
              int i = kept[q];
              xi[i] += fre(lk[q]) * (sc[i] / skk) * x;
            }
          }
        }
        // Schur update a_ij -= l_ik d conj(l_jk); each row has one owner
        // thread.  Neighbours whose L entry was dropped only lose column k.
        for (size_t q = 0; q < kept.size(); ++q) inkept[kept[q]] = 1;
        nbr.clear();
        for (auto& e : A.rows[k])
          if (!inkept[e.col] && state[e.col] != 1) nbr.push_back(e.col);
        const int nkept = (int)kept.size();
        pool.run(nkept + (int)nbr.size(), [&](int tid, int q) {
          if (q >= nkept) {
            remove_col(nbr[q - nkept], k);
            return;
          }
          // One pass over row i maps its columns (and finds column k); the
          // updates, the appended fill and the removal of column k are those
          // of a slot array that is set, used and cleared per row.
          PosStamp* ps = tpos[tid].data();
          uint32_t stamp = ++tstamp[tid];
          if (stamp == 0) {  // the counter wrapped: clear the map once
            for (int c = 0; c < n; ++c) ps[c] = PosStamp{0u, -1};
            stamp = tstamp[tid] = 1;
          }
          int i = kept[q];
          auto& row = A.rows[i];
          size_t pk = SIZE_MAX;
          for (size_t t = 0; t < row.size(); ++t) {
            const int c = row[t].col;
            ps[c] = PosStamp{stamp, (int)t};
            if (c == k && pk == SIZE_MAX) pk = t;
          }
          T li = lk[q];
          A.diag[i] -= T(fre(li * d * fcj(li)));
          const T lid = li * d;  // u = li * d * conj(l_j), evaluated left to right
          for (size_t t = 0; t < kept.size(); ++t) {
            if (t == (size_t)q) continue;
            int j = kept[t];
            T u = lid * fcj(lk[t]);
            if (ps[j].stamp == stamp) row[ps[j].pos].val -= u;
            else if (fab(u) * sc[i] * sc[j] > lvl_dropS) {
              row.push_back({j, -u});
              ps[j] = PosStamp{stamp, (int)row.size() - 1};
            }
          }
          if (pk != SIZE_MAX) {
            row[pk] = row.back();
            row.pop_back();
          }
        });
        for (int i : kept) {
          dlev[i] = std::max(dlev[i], dlev[k] + 1);
          inkept[i] = 0;
        }
        pos[k] = (int)order.size();
        order.push_back(k);
        blk[pos[k]] = 1;
        dinv[pos[k]] = T(1) / d;
        for (size_t q = 0; q < kept.size(); ++q) { crow.push_back(kept[q]); cval.push_back(lk[q]); }
        colptr.push_back((int64_t)crow.size());
        state[k] = 1;
        A.rows[k].clear();
        A.rows[k].shrink_to_fit();
        for (auto& e : kept) (void)e;
        accepted_here++;
      } else if (piv == 2) {
        int j = jp;
        T akj = T(0);
        for (auto& e : A.rows[k])
          if (e.col == j) { akj = e.val; break; }  // A(k,j)
        T dkk = A.diag[k], djj = A.diag[j];
        T det = dkk * djj - akj * fcj(akj);
        double sj = sc[j];
        double dets = fab(det) * skk * skk * sj * sj, offs = fab(akj) * skk * sj;
        bool ok = dets > 1e-3 * offs * offs && fab(det) > 0;
        // gather A(i,k) and A(i,j) for the union of neighbours
        std::vector<int>& nb = kept;
        nb.clear();
        for (auto& e : A.rows[k])
          if (e.col != j && state[e.col] != 1 && slot[e.col] < 0) { slot[e.col] = (int)nb.size(); nb.push_back(e.col); }
        for (auto& e : A.rows[j])
          if (e.col != k && state[e.col] != 1 && slot[e.col] < 0) { slot[e.col] = (int)nb.size(); nb.push_back(e.col); }
        std::vector<T> aik(nb.size(), T(0)), aij(nb.size(), T(0));
        for (auto& e : A.rows[k])
          if (e.col != j && state[e.col] != 1) aik[slot[e.col]] = fcj(e.val);
        for (auto& e : A.rows[j])
          if (e.col != k && state[e.col] != 1) aij[slot[e.col]] = fcj(e.val);
        for (int c : nb) slot[c] = -1;
        // D^{-1} = (1/det) [djj, -akj; -conj(akj), dkk]
        T i00 = djj / det, i11 = dkk / det, i01 = -akj / det;  // (k,j) entry
        T i10 = fcj(i01);
        lk.assign(nb.size(), T(0));
        lj.assign(nb.size(), T(0));
        double lmax = 0;
        for (size_t q = 0; q < nb.size(); ++q) {
          lk[q] = aik[q] * i00 + aij[q] * i10;
          lj[q] = aik[q] * i01 + aij[q] * i11;
          lmax = std::max(lmax, std::max(fab(lk[q]) * sc[nb[q]] / skk, fab(lj[q]) * sc[nb[q]] / sj));
        }
        if (!last && (!ok || lmax > kappa)) {
          state[k] = 2;
          deferred.push_back(k);
          continue;
        }
        if (last && !(fab(det) > 0)) return (int)order.size() + 1;
        double nxk = last ? 1.0 : nu_of(k), nxj = last ? 1.0 : nu_of(j);
        const bool crule = prm.drop_rule == 1 && !last;
        double thk = 0, thj = 0;
        if (crule) {
          double mk = 0, mj = 0;
          for (size_t q = 0; q < nb.size(); ++q) {
            mk = std::max(mk, fab(lk[q]) * sc[nb[q]] / skk);
            mj = std::max(mj, fab(lj[q]) * sc[nb[q]] / sj);
          }
          const double bd = std::max({fab(dkk) * skk * skk, fab(djj) * sj * sj, fab(akj) * skk * sj});
          thk = crule_thr(nxk, bd, mk);
          thj = crule_thr(nxj, bd, mj);
        }
        // dropping per entry
        std::vector<char> keepk(nb.size()), keepj(nb.size());
        for (size_t q = 0; q < nb.size(); ++q) {
          keepk[q] = crule ? fab(lk[q]) * sc[nb[q]] / skk > thk : fab(lk[q]) * sc[nb[q]] / skk * nxk > lvl_droptol;
          keepj[q] = crule ? fab(lj[q]) * sc[nb[q]] / sj > thj : fab(lj[q]) * sc[nb[q]] / sj * nxj > lvl_droptol;
          if (!keepk[q]) lk[q] = T(0);
          if (!keepj[q]) lj[q] = T(0);
        }
        if (!last && prm.lookahead) {
          bool over = false;
          if (is_cplx) {
            cplx xk = (std::abs(xic[k]) > 0) ? -xic[k] / std::abs(xic[k]) * (1 + std::abs(xic[k])) : cplx(1);
            cplx xj = (std::abs(xic[j]) > 0) ? -xic[j] / std::abs(xic[j]) * (1 + std::abs(xic[j])) : cplx(1);
            for (size_t q = 0; q < nb.size() && !over; ++q) {
              const int i = nb[q];
              over = std::abs(xic[i] + cplx(lk[q] * T(sc[i] / skk)) * xk + cplx(lj[q] * T(sc[i] / sj)) * xj) > kappa;
            }
          } else {
            double xk = (xi[k] != 0) ? -(xi[k] / std::fabs(xi[k])) * (1 + std::fabs(xi[k])) : 1.0;
            double xj = (xi[j] != 0) ? -(xi[j] / std::fabs(xi[j])) * (1 + std::fabs(xi[j])) : 1.0;
            for (size_t q = 0; q < nb.size() && !over; ++q) {
              const int i = nb[q];
              over = std::fabs(xi[i] + fre(lk[q]) * (sc[i] / skk) * xk + fre(lj[q]) * (sc[i] / sj) * xj) > kappa;
            }
          }
          if (over) {
            state[k] = 2;
            deferred.push_back(k);
            continue;
          }
        }
        if (!last) {
          if (is_cplx) {
            cplx xk = (std::abs(xic[k]) > 0) ? -xic[k] / std::abs(xic[k]) * (1 + std::abs(xic[k])) : cplx(1);
            cplx xj = (std::abs(xic[j]) > 0) ? -xic[j] / std::abs(xic[j]) * (1 + std::abs(xic[j])) : cplx(1);
            for (size_t q = 0; q < nb.size(); ++q) {
              int i = nb[q];
              xic[i] += cplx(lk[q] * T(sc[i] / skk)) * xk + cplx(lj[q] * T(sc[i] / sj)) * xj;
            }
          } else {
            double xk = (xi[k] != 0) ? -(xi[k] / std::fabs(xi[k])) * (1 + std::fabs(xi[k])) : 1.0;
            double xj = (xi[j] != 0) ? -(xi[j] / std::fabs(xi[j])) * (1 + std::fabs(xi[j])) : 1.0;
            for (size_t q = 0; q < nb.size(); ++q) {
              int i = nb[q];
              xi[i] += fre(lk[q]) * (sc[i] / skk) * xk + fre(lj[q]) * (sc[i] / sj) * xj;
            }
          }
        }
        // t_l = D [conj(l_lk); conj(l_lj)] ; update_il = l_ik t_l0 + l_ij t_l1
        std::vector<int> act;
        for (size_t q = 0; q < nb.size(); ++q)
          if (keepk[q] || keepj[q]) act.push_back((int)q);
        pool.run((int)act.size(), [&](int tid, int qq) {
          PosStamp* ps = tpos[tid].data();
          uint32_t stamp = ++tstamp[tid];
          if (stamp == 0) {
            for (int c = 0; c < n; ++c) ps[c] = PosStamp{0u, -1};
            stamp = tstamp[tid] = 1;
          }
          const int qa = act[qq];
          int i = nb[qa];
          auto& row = A.rows[i];
          for (size_t t = 0; t < row.size(); ++t) ps[row[t].col] = PosStamp{stamp, (int)t};
          for (int ta : act) {
            int l = nb[ta];
            T c0 = fcj(lk[ta]), c1 = fcj(lj[ta]);
            T t0 = dkk * c0 + akj * c1, t1 = fcj(akj) * c0 + djj * c1;
            T u = lk[qa] * t0 + lj[qa] * t1;
            if (l == i) { A.diag[i] -= T(fre(u)); continue; }
            if (ps[l].stamp == stamp) row[ps[l].pos].val -= u;
            else if (fab(u) * sc[i] * sc[l] > lvl_dropS) {
              row.push_back({l, -u});
              ps[l] = PosStamp{stamp, (int)row.size() - 1};
            }
          }
        });
        {
          int lv = std::max(dlev[k], dlev[j]) + 1;
          for (size_t q = 0; q < nb.size(); ++q)
            if (keepk[q] || keepj[q]) dlev[nb[q]] = std::max(dlev[nb[q]], lv);
        }
        for (auto& e : A.rows[k]) if (e.col != j) remove_col(e.col, k);
        for (auto& e : A.rows[j]) if (e.col != k) remove_col(e.col, j);
        Q.remove(j);
        pos[k] = (int)order.size();
        order.push_back(k);
        pos[j] = (int)order.size();
        order.push_back(j);
        blk[pos[k]] = 2;
        blk[pos[j]] = -2;
        dinv[pos[k]] = i00;
        dinv[pos[j]] = i11;
        doff[pos[k]] = i01;
        for (size_t q = 0; q < nb.size(); ++q)
          if (keepk[q]) { crow.push_back(nb[q]); cval.push_back(lk[q]); }
        colptr.push_back((int64_t)crow.size());
        for (size_t q = 0; q < nb.size(); ++q)
          if (keepj[q]) { crow.push_back(nb[q]); cval.push_back(lj[q]); }
        colptr.push_back((int64_t)crow.size());
        state[k] = 1;
        state[j] = 1;
        A.rows[k].clear();
        A.rows[k].shrink_to_fit();
        A.rows[j].clear();
        A.rows[j].shrink_to_fit();
        accepted_here += 2;
      } else {
        state[k] = 2;
        deferred.push_back(k);
        continue;
      }
      if (over_mem()) return -3;
      // degree updates of the touched rows
      for (int i : kept)
        if (state[i] == 0) Q.update(i, qkey(i));
    }
    if (prm.verbose) {
      const double now = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
      std::fprintf(stderr, "ildlc level %d: %d rows (%s%s), %d accepted, %lld level entries, L %lld, %.1f s\n",
                   level, nl, last ? "last" : "deferring", dense_lvl ? ", dense" : "", accepted_here,
                   (long long)level_entries, (long long)crow.size(), now - t_level0);
      t_level0 = now;
    }
    if (fform) {
      for (auto& t : snap) {
        if (state[t.r] == 1 && state[t.c] == 2) fent.push_back(t);
        else if (state[t.r] == 2 && state[t.c] == 1) fent.push_back({t.c, t.r, fcj(t.v)});
      }
      snap.clear();
      snap.shrink_to_fit();
      // stored: the L entries between this level's accepted rows
      for (int64_t q = crow_lvl0; q < (int64_t)crow.size(); ++q)
        if (state[crow[q]] == 1) stored_done++;
      if (stored_done + (int64_t)fent.size() + n > memcap) return -3;
    }
    level++;
    if (deferred.empty()) break;
    if (!last && (double)accepted_here < prm.min_progress * nl) last = true;
    level_nodes = deferred;
  }
  F.level_start.push_back(n);
  // convert the column-wise L to CSR rows in elimination order
  F.perm = order;
  F.blk = blk;
  F.dinv = dinv;
  F.doff = doff;
  F.coupling = fform ? 1 : 0;
  // coupling 1 keeps only the entries inside a level (column step p and its rows in the same level)
  auto keep_entry = [&](int p, int r) { return !fform || node_level[order[p]] == node_level[order[r]]; };
  std::vector<int64_t> rc(n + 1, 0);
  for (int p = 0; p < n; ++p)
    for (int64_t q = colptr[p]; q < colptr[p + 1]; ++q)
      if (keep_entry(p, pos[crow[q]])) rc[pos[crow[q]] + 1]++;
  for (int p = 0; p < n; ++p) rc[p + 1] += rc[p];
  F.lp = rc;
  F.li.assign(rc[n], 0);
  F.lx.assign(rc[n], T(0));
  std::vector<int64_t> fillp(rc.begin(), rc.end() - 1);
  for (int p = 0; p < n; ++p)
    for (int64_t q = colptr[p]; q < colptr[p + 1]; ++q) {
      int r = pos[crow[q]];
      if (!keep_entry(p, r)) continue;
      F.li[fillp[r]] = p;
      F.lx[fillp[r]] = cval[q];
      fillp[r]++;
    }
  if (fform) {
    // F in CSR over elimination steps, columns ascending within a row
    F.fp.assign(n + 1, 0);
    for (auto& t : fent) F.fp[pos[t.r] + 1]++;
    for (int p = 0; p < n; ++p) F.fp[p + 1] += F.fp[p];
    F.fi.assign(fent.size(), 0);
    F.fx.assign(fent.size(), T(0));
    std::vector<int64_t> fq(F.fp.begin(), F.fp.end() - 1);
    for (auto& t : fent) {
      const int64_t q = fq[pos[t.r]]++;
      F.fi[q] = pos[t.c];
      F.fx[q] = t.v;
    }
    for (int p = 0; p < n; ++p) {
      std::vector<std::pair<int, T>> row;
      for (int64_t q = F.fp[p]; q < F.fp[p + 1]; ++q) row.push_back({F.fi[q], F.fx[q]});
      std::sort(row.begin(), row.end(), [](const std::pair<int, T>& x, const std::pair<int, T>& y) {
        return x.first < y.first;
      });
      for (size_t t = 0; t < row.size(); ++t) {
        F.fi[F.fp[p] + t] = row[t].first;
        F.fx[F.fp[p] + t] = row[t].second;
      }
    }
  }
  // |D|^{-1} (SPD conversion) and the count of negative eigenvalues of D
  F.ainv.assign(n, T(0));
  F.aoff.assign(n, T(0));
  F.nneg = 0;
  for (int p = 0; p < n; ++p) {
    if (F.blk[p] == 1) {
      double v = fre(F.dinv[p]);
      if (v < 0) F.nneg++;
      F.ainv[p] = T(std::fabs(v));
    } else if (F.blk[p] == 2) {
      // eigen-decomposition of the Hermitian 2x2 inverse block [a b; conj(b) c]
      double a = fre(F.dinv[p]), c = fre(F.dinv[p + 1]);
      T bo = F.doff[p];
      double bb = fab(bo);
      double mid = 0.5 * (a + c), rad = std::sqrt(0.25 * (a - c) * (a - c) + bb * bb);
      double l1 = mid + rad, l2 = mid - rad;
      if (l1 < 0) F.nneg++;
      if (l2 < 0) F.nneg++;
      // |M| = M * sign-matrix: |M| = (|l1|+|l2|)/2 I + (|l1|-|l2|)/(2 rad) (M - mid I)
      double al1 = std::fabs(l1), al2 = std::fabs(l2);
      if (rad > 0) {
        double s0 = 0.5 * (al1 + al2), s1 = 0.5 * (al1 - al2) / rad;
        F.ainv[p] = T(s0 + s1 * (a - mid));
        F.ainv[p + 1] = T(s0 + s1 * (c - mid));
        F.aoff[p] = T(s1) * bo;
      } else {
        F.ainv[p] = T(al1);
        F.ainv[p + 1] = T(al1);
        F.aoff[p] = T(0);
      }
    }
  }
  return 0;
}

// Forward and backward level schedules of the unit L of a factor: rows of the
// same level have no dependency on each other.  fwd_rows lists the rows level
// by level (fwd_ptr), bwd_rows likewise for L^H.
template <class T>
void ildlc_levels(const IldlcFactor<T>& F, std::vector<int>& fwd_ptr, std::vector<int>& fwd_rows,
                  std::vector<int>& bwd_ptr, std::vector<int>& bwd_rows) {
  const int n = F.n;
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int p = 0; p < n; ++p) {
    int m = 0;
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) m = std::max(m, lev[F.li[q]] + 1);
    lev[p] = m;
    nlev = std::max(nlev, m + 1);
  }
  auto bucket = [&](const std::vector<int>& lv, int nl, std::vector<int>& ptr, std::vector<int>& rows) {
    ptr.assign(nl + 1, 0);
    for (int p = 0; p < n; ++p) ptr[lv[p] + 1]++;
    for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
    rows.assign(n, 0);
    std::vector<int> f(ptr.begin(), ptr.end() - 1);
    for (int p = 0; p < n; ++p) rows[f[lv[p]]++] = p;
  };
  bucket(lev, n ? nlev : 0, fwd_ptr, fwd_rows);
  // backward: column p of L (rows r > p with L(r,p) != 0) must be final first
  std::vector<int> blev(n, 0);
  int nb = 0;
  for (int p = n - 1; p >= 0; --p) {
    // blev[p] already holds max over dependents via the push below
    nb = std::max(nb, blev[p] + 1);
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) {
      int c = F.li[q];
      blev[c] = std::max(blev[c], blev[p] + 1);
    }
  }
  bucket(blev, n ? nb : 0, bwd_ptr, bwd_rows);
}

}  // namespace jdg
