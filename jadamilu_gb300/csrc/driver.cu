// Preconditioner-aware driver and the Fortran-callable C ABI.
//
// Follows the reference's PJDRVCOM (src/jd/JDaux.F:5-544), PJDINIT
// (:549-1325) and PJDCLEANUP1 (:1332-1381): shift selection, factorisation
// with automatic retries, SPD conversion, adaptive re-factorisation during the
// iteration, and the suggested SHIFT/DROPTOL on exit.  The global state of the
// reference's COMMON blocks becomes one `Global` object per arithmetic (real,
// complex), which keeps the drop-in contract of one solve per precision at a
// time, including the ICNTL(2) = -1/-2 reuse of the previous preconditioner.
//
// Reverse communication (DPJDREVCOM/DJDREVCOM and the _GEP forms) runs the
// solver on a worker thread that hands each matvec / preconditioner request
// back to the caller's thread; all CUDA work stays on the worker.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <limits>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>

#include "devjd.cuh"
#include "ildlc.hpp"
#include "tail_inverse.hpp"
#include "block_plan.hpp"
#include "../../include/jadamilu_gb300.h"

namespace jdg {

static double wall() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// --------------------------------------------------------- device matrix ----
template <class T, class H>
void build_sell(int n, const int* ia, const int* ja, const H* a, SellMatrix<T>& M, cudaStream_t st) {
  std::vector<int> cnt(n, 0);
  for (int i = 0; i < n; ++i)
    for (int p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
      int j = ja[p] - 1;
      cnt[i]++;
      if (j != i) cnt[j]++;
    }
  std::vector<int64_t> rp(n + 1, 0);
  for (int i = 0; i < n; ++i) rp[i + 1] = rp[i] + cnt[i];
  std::vector<int> ci(rp[n]);
  std::vector<T> cv(rp[n]);
  std::vector<int64_t> fp(rp.begin(), rp.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
      int j = ja[p] - 1;
      H v = a[p];
      ci[fp[i]] = j;
      cv[fp[i]++] = todev(v);
      if (j != i) {
        ci[fp[j]] = i;
        cv[fp[j]++] = todev(jdd::cj(v));
      }
    }
  const int ns = (n + 31) / 32;
  std::vector<int64_t> sp(ns + 1, 0);
  for (int s = 0; s < ns; ++s) {
    int w = 0;
    for (int r = s * 32; r < std::min(n, s * 32 + 32); ++r) w = std::max(w, cnt[r]);
    sp[s + 1] = sp[s] + (int64_t)w * 32;
  }
  std::vector<int> scol(sp[ns]);
  std::vector<T> sval(sp[ns], T(0));
  for (int s = 0; s < ns; ++s) {
    int w = (int)((sp[s + 1] - sp[s]) / 32);
    for (int lane = 0; lane < 32; ++lane) {
      int r = s * 32 + lane;
      for (int q = 0; q < w; ++q) {
        int64_t dst = sp[s] + (int64_t)q * 32 + lane;
        if (r < n && q < cnt[r]) {
          scol[dst] = ci[rp[r] + q];
          sval[dst] = cv[rp[r] + q];
        } else {
          scol[dst] = r < n ? r : 0;
          sval[dst] = T(0);
        }
      }
    }
  }
  if (M.sptr) { cudaFree(M.sptr); cudaFree(M.col); cudaFree(M.val); }
  M.n = n;
  M.nslices = ns;
  M.nnz = rp[n];
  M.stored = sp[ns];
  CK(cudaMalloc(&M.sptr, sizeof(int64_t) * (ns + 1)));
  CK(cudaMalloc(&M.col, sizeof(int) * std::max<int64_t>(1, sp[ns])));
  CK(cudaMalloc(&M.val, sizeof(T) * std::max<int64_t>(1, sp[ns])));
  CK(cudaMemcpyAsync(M.sptr, sp.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(M.col, scol.data(), sizeof(int) * sp[ns], cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(M.val, sval.data(), sizeof(T) * sp[ns], cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
}
template <class T> void free_sell(SellMatrix<T>& M) {
  if (M.sptr) { cudaFree(M.sptr); cudaFree(M.col); cudaFree(M.val); }
  M = SellMatrix<T>();
}

// --------------------------------------------------------- device factor ----
template <class S> struct StoreOf;
template <> struct StoreOf<double> { static double f(double v) { return v; } };
template <> struct StoreOf<float> { static float f(double v) { return (float)v; } };
template <> struct StoreOf<__nv_bfloat16> { static __nv_bfloat16 f(double v) { return __float2bfloat16((float)v); } };
template <> struct StoreOf<zc> { static zc f(std::complex<double> v) { return zc(v.real(), v.imag()); } };
template <> struct StoreOf<cc> { static cc f(std::complex<double> v) { return cc((float)v.real(), (float)v.imag()); } };
template <> struct StoreOf<bc> {
  static bc f(std::complex<double> v) { return bc{__float2bfloat16((float)v.real()), __float2bfloat16((float)v.imag())}; }
};

template <class S> void free_factor(DevFactor<S>& F) {
  void* ps[] = {F.orig, F.lp,  F.li,  F.lx,  F.up,  F.ui,  F.ux,    F.brows, F.blk,   F.partner, F.dv,
                F.dof,  F.av,  F.aof, F.y,   F.dfptr, F.dbptr, F.rhs_in, F.sol_out, F.tep, F.tei, F.tev,
                F.tip,  F.tii, F.tiv, F.dtfptr, F.tbp, F.tbi, F.tbv, F.dtbptr, F.tbrows,
                F.part, F.xb, F.perm, F.fpp, F.fpi, F.fpx, F.fhp, F.fhi, F.fhx, F.cy, F.cyb, F.ct};
  for (void* p : ps)
    if (p) cudaFree(p);
  for (auto& L : F.lev) free_factor(L);
  for (auto& B : F.blocks) {
    void* bs[] = {B.ep, B.ei, B.ev, B.bp, B.bi, B.bv, B.tf, B.tb, B.itf, B.itb, B.irf, B.irb};
    for (void* p : bs)
      if (p) cudaFree(p);
  }
  for (auto& g : F.graph)
    if (g) cudaGraphExecDestroy(g);
  F = DevFactor<S>();
}

struct Options {
  double depth_weight = 64.0;
  int verbose = 0;
  int dense_tail = 1;          // solve the deepest levels with their explicit inverse
  int dense_max = 32768;       // at most this many rows in the dense tail
  double dense_min_saving = 100e-6;  // modelled seconds per application the dense blocks must save
  double plan_launch_us = 4.0;       // the block planner's cost of one launch (microseconds)
  double plan_tile_gbs = 5000.0;     // and its streaming rate of L entries and tiles (GB/s)
  double drop_schur = -1.0;    // IldlcParams::droptol_schur (negative: its default rule)
  int apply_graph = 0;         // jdgpu_dildl_apply through the captured graph
  int fuse_inner = 1;          // inner iterations read their scalars back once (library operators only)
  int revcom_device = 0;       // reverse-communication requests are served on the device copy of X
  int matching = 0;            // first factor level decides with the maximum-product matching scale
  // factor form (IldlcParams) from coupled_min_n rows on: the Schur-
  // contribution drop rule, look-ahead pivot deferral and an exact last level
  // once a level's matrix is a third full; one global L (coupling 0, one
  // sweep each way) or, with coupling 1, per-level coupling blocks (less
  // memory, two B-solves per level)
  int coupling = 0;
  int drop_rule = 1;
  int lookahead = 1;
  double last_droptol = 0.0;
  double last_fill = 1.0 / 3.0;
  int coupled_min_n = 4096;    // smaller matrices keep the plain factor (drop rule 0, no look-ahead)
  // a solve takes that form only when its ISEARCH is at least this: 2, the
  // interior eigenvalues of an indefinite shifted matrix (ISEARCH 0 and 1
  // factor a matrix shifted below or near the lower end of the spectrum)
  int large_form_isearch = 2;
  int factor_verbose = 0;
  int tri_cluster = 8;         // CTAs per cluster of the tile product: 8, or 16 where the GPU allows it
  int dense_min_rows = -1;     // IldlcParams::dense_min_rows (negative: its default)
};
static Options g_opt;

// the tile product's cluster size for a factor uploaded now (16 only where
// the current device runs clusters of that non-portable size)
template <class S> static int tile_cluster() {
  if (g_opt.tri_cluster != 16) return 8;
  return k::tri_cluster16_ok<S, typename Arith<S>::type>() ? 16 : 8;
}

// the factor options of this library on top of the caller's droptol/condest/mem;
// isearch: the solve's ISEARCH (2 for the factor-only and gradient entry points)
static void factor_options(IldlcParams& p, int n, int isearch = 2) {
  p.depth_weight = g_opt.depth_weight;
  p.droptol_schur = g_opt.drop_schur;
  p.matching = g_opt.matching;
  p.verbose = g_opt.factor_verbose;
  if (g_opt.dense_min_rows >= 0) p.dense_min_rows = g_opt.dense_min_rows;
  if (n >= g_opt.coupled_min_n && isearch >= g_opt.large_form_isearch) {
    p.coupling = g_opt.coupling;
    p.drop_rule = g_opt.drop_rule;
    p.last_droptol = g_opt.last_droptol;
    p.last_fill = g_opt.last_fill;
    p.lookahead = g_opt.lookahead;
  }
}

// device memory for the factor arrays: cudaMalloc unless the caller supplies
// another source
struct DeviceMalloc {
  void* operator()(size_t bytes) const {
    void* p = nullptr;
    CK(cudaMalloc(&p, bytes));
    return p;
  }
};

template <class S, class H, class Alloc>
void upload_coupled(const IldlcFactor<H>& F, DevFactor<S>& D, cudaStream_t st, Alloc alloc, bool graph_io);

template <class S, class H, class Alloc = DeviceMalloc>
void upload_factor(const IldlcFactor<H>& F, DevFactor<S>& D, cudaStream_t st, Alloc alloc = Alloc(),
                   bool graph_io = true) {
  free_factor(D);
  if (F.coupling == 1) {
    upload_coupled(F, D, st, alloc, graph_io);
    return;
  }
  const int n = F.n;
  // forward levels over elimination steps; solve numbering s = level order
  std::vector<int> flev(n, 0);
  int nfl = n ? 1 : 0;
  for (int p = 0; p < n; ++p) {
    int m = 0;
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q) m = std::max(m, flev[F.li[q]] + 1);
    flev[p] = m;
    nfl = std::max(nfl, m + 1);
  }
  std::vector<int> fptr(nfl + 1, 0);
  for (int p = 0; p < n; ++p) fptr[flev[p] + 1]++;
  for (int l = 0; l < nfl; ++l) fptr[l + 1] += fptr[l];
  std::vector<int> snum(n), pof(n);
  {
    std::vector<int> f(fptr.begin(), fptr.end() - 1);
    for (int p = 0; p < n; ++p) {
      int s = f[flev[p]]++;
      snum[p] = s;
      pof[s] = p;
    }
  }
  // tail: the deepest run of narrow levels, as long as its part of y fits in
  // shared memory
  using A = typename DevFactor<S>::A;
  // per tail row: its y entry, a row pointer, a level pointer and a row index
  const int tail_max = std::min<int>(16384, (int)((200 * 1024) / (sizeof(A) + 12)));
  // forward rows in s numbering
  std::vector<int> orig(n);
  std::vector<int64_t> lp(n + 1, 0);
  for (int s = 0; s < n; ++s) lp[s + 1] = lp[s] + (F.lp[pof[s] + 1] - F.lp[pof[s]]);
  std::vector<int> li(lp[n]);
  std::vector<S> lx(lp[n]);
  std::vector<H> lxh(lp[n]);
  std::vector<int64_t> up(n + 1, 0);
  for (int s = 0; s < n; ++s) {
    int p = pof[s];
    orig[s] = F.perm[p];
    int64_t o = lp[s];
    for (int64_t q = F.lp[p]; q < F.lp[p + 1]; ++q, ++o) {
      li[o] = snum[F.li[q]];
      lxh[o] = F.lx[q];
      lx[o] = StoreOf<S>::f(F.lx[q]);
      up[li[o] + 1]++;
    }
  }
  for (int s = 0; s < n; ++s) up[s + 1] += up[s];
  std::vector<int> ui(up[n]);
  std::vector<S> ux(up[n]);
  {
    std::vector<int64_t> fu(up.begin(), up.end() - 1);
    for (int s = 0; s < n; ++s)
      for (int64_t q = lp[s]; q < lp[s + 1]; ++q) {
        int c = li[q];
        ui[fu[c]] = s;
        ux[fu[c]++] = StoreOf<S>::f(jdd::cj(lxh[q]));
      }
  }
  // rows from s_tail on: dense blocks (plan_dense_blocks), or with the
  // dense_tail option off the deepest run of narrow levels in one CTA
  const bool dense_opt = g_opt.dense_tail != 0 && n > 0;
  std::vector<BlockGroup> groups;
  int Lt = nfl;
  if (dense_opt) {
    std::vector<int64_t> ent_f(nfl, 0), ent_b(nfl, 0);
    for (int l = 0; l < nfl; ++l)
      for (int s = fptr[l]; s < fptr[l + 1]; ++s) {
        ent_f[l] += lp[s + 1] - lp[s];
        ent_b[l] += up[s + 1] - up[s];
      }
    groups = plan_dense_blocks(fptr, ent_f, ent_b, sizeof(S), g_opt.dense_max, g_opt.dense_min_saving,
                               g_opt.plan_launch_us * 1e-6, g_opt.plan_launch_us * 1e-6, g_opt.plan_tile_gbs * 1e9);
    if (!groups.empty()) Lt = groups[0].a;
  } else {
    int acc_rows = 0;
    while (Lt > 1) {
      int r = fptr[Lt] - fptr[Lt - 1];
      if (r > 2048 || acc_rows + r > tail_max) break;
      acc_rows += r;
      --Lt;
    }
  }
  const bool dense = !groups.empty();
  const int s_tail = fptr[Lt];
  const int m_tail = n - s_tail;
  // the single-CTA tail arrays (level path only; empty with dense blocks)
  const int m_lv = dense ? 0 : m_tail;
  // forward tail split into external / internal entries
  std::vector<int64_t> tep(m_lv + 1, 0), tip(m_lv + 1, 0);
  for (int t = 0; t < m_lv; ++t) {
    int s = s_tail + t;
    int64_t ne = 0, ni = 0;
    for (int64_t q = lp[s]; q < lp[s + 1]; ++q) (li[q] < s_tail ? ne : ni)++;
    tep[t + 1] = tep[t] + ne;
    tip[t + 1] = tip[t] + ni;
  }
  std::vector<int> tei(tep[m_lv]), tii(tip[m_lv]);
  std::vector<S> tev(tep[m_lv]), tiv(tip[m_lv]);
  for (int t = 0; t < m_lv; ++t) {
    int s = s_tail + t;
    int64_t oe = tep[t], oi = tip[t];
    for (int64_t q = lp[s]; q < lp[s + 1]; ++q) {
      if (li[q] < s_tail) { tei[oe] = li[q]; tev[oe++] = lx[q]; }
      else { tii[oi] = li[q] - s_tail; tiv[oi++] = lx[q]; }
    }
  }
  std::vector<int> tfptr;
  for (int l = Lt; l <= nfl; ++l) tfptr.push_back(fptr[l] - s_tail);
  // backward: tail rows first (all their dependents are tail rows), then the
  // bulk rows level by level (dependencies on tail rows are already final)
  std::vector<int> blev(n, 0);
  int nbl = 0, ntl = 0;
  for (int s = n - 1; s >= 0; --s) {
    int m = 0;
    const bool tail = s >= s_tail;
    for (int64_t q = up[s]; q < up[s + 1]; ++q) {
      int r = ui[q];
      if (tail || r < s_tail) m = std::max(m, blev[r] + 1);
    }
    blev[s] = m;
    if (tail) ntl = std::max(ntl, m + 1);
    else nbl = std::max(nbl, m + 1);
  }
  std::vector<int> bptr(nbl + 1, 0), brs(std::max(0, s_tail));
  for (int s = 0; s < s_tail; ++s) bptr[blev[s] + 1]++;
  for (int l = 0; l < nbl; ++l) bptr[l + 1] += bptr[l];
  {
    std::vector<int> f(bptr.begin(), bptr.end() - 1);
    for (int s = 0; s < s_tail; ++s) brs[f[blev[s]]++] = s;
  }
  std::vector<int> tbptr(ntl + 1, 0), tbrows(m_lv);
  for (int t = 0; t < m_lv; ++t) tbptr[blev[s_tail + t] + 1]++;
  for (int l = 0; l < ntl; ++l) tbptr[l + 1] += tbptr[l];
  {
    std::vector<int> f(tbptr.begin(), tbptr.end() - 1);
    for (int t = 0; t < m_lv; ++t) tbrows[f[blev[s_tail + t]]++] = t;
  }
  std::vector<int64_t> tbp(m_lv + 1, 0);
  for (int t = 0; t < m_lv; ++t) tbp[t + 1] = tbp[t] + (up[s_tail + t + 1] - up[s_tail + t]);
  std::vector<int> tbi(tbp[m_lv]);
  std::vector<S> tbv(tbp[m_lv]);
  for (int t = 0; t < m_lv; ++t) {
    int64_t o = tbp[t];
    for (int64_t q = up[s_tail + t]; q < up[s_tail + t + 1]; ++q, ++o) {
      tbi[o] = ui[q] - s_tail;
      tbv[o] = ux[q];
    }
  }
  std::vector<signed char> blk(n);
  std::vector<int> partner(n, -1);
  std::vector<S> dv(n), dof(n), av(n), aof(n);
  for (int s = 0; s < n; ++s) {
    int p = pof[s];
    blk[s] = F.blk[p];
    dv[s] = StoreOf<S>::f(F.dinv[p]);
    dof[s] = StoreOf<S>::f(F.doff[p]);
    av[s] = StoreOf<S>::f(F.ainv[p]);
    aof[s] = StoreOf<S>::f(F.aoff[p]);
    if (F.blk[p] == 2) {
      partner[s] = snum[p + 1];
      partner[snum[p + 1]] = s;
    }
  }
  D.n = n;
  D.nnz_l = lp[n];
  D.fptr.assign(fptr.begin(), fptr.begin() + Lt + 1);
  D.bptr = bptr;
  D.s_tail = s_tail;
  D.m_tail = m_tail;
  D.tfptr = tfptr;
  D.tbptr = tbptr;
  auto up_ = [&](auto*& dst, const auto& src) {
    using E = typename std::remove_reference<decltype(src)>::type::value_type;
    size_t bytes = sizeof(E) * std::max<size_t>(1, src.size());
    dst = (std::remove_reference_t<decltype(dst)>)alloc(bytes);
    if (!src.empty()) CK(cudaMemcpyAsync(dst, src.data(), sizeof(E) * src.size(), cudaMemcpyHostToDevice, st));
  };
  up_(D.orig, orig);
  up_(D.lp, lp);
  up_(D.li, li);
  up_(D.lx, lx);
  up_(D.up, up);
  up_(D.ui, ui);
  up_(D.ux, ux);
  up_(D.brows, brs);
  up_(D.blk, blk);
  up_(D.partner, partner);
  up_(D.dv, dv);
  up_(D.dof, dof);
  up_(D.av, av);
  up_(D.aof, aof);
  up_(D.dfptr, D.fptr);
  up_(D.dbptr, bptr);
  up_(D.tep, tep);
  up_(D.tei, tei);
  up_(D.tev, tev);
  up_(D.tip, tip);
  up_(D.tii, tii);
  up_(D.tiv, tiv);
  up_(D.dtfptr, tfptr);
  up_(D.tbp, tbp);
  up_(D.tbi, tbi);
  up_(D.tbv, tbv);
  up_(D.dtbptr, tbptr);
  up_(D.tbrows, tbrows);
  // dense blocks: external entries of both sweeps and, for dense groups, the
  // explicit inverse of the diagonal block from the internal entries in host
  // precision; each block is uploaded as soon as it is built
  D.sweep_entries = dense ? lp[s_tail] + up[s_tail] : 2 * lp[n];
  D.tile_bytes = 0;
  size_t max_items = 0;
  const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  for (const auto& gr : groups) {
    DenseBlk<S> B;
    B.s0 = fptr[gr.a];
    B.m = fptr[gr.b] - B.s0;
    std::vector<int64_t> ep(B.m + 1, 0), bp(B.m + 1, 0), ip(B.m + 1, 0);
    std::vector<int> ei, bi, ii;
    std::vector<S> ev, bv;
    std::vector<H> iv;
    for (int t = 0; t < B.m; ++t) {
      const int s = B.s0 + t;
      for (int64_t q = lp[s]; q < lp[s + 1]; ++q) {
        if (li[q] < B.s0) {
          ei.push_back(li[q]);
          ev.push_back(lx[q]);
        } else {
          ii.push_back(li[q] - B.s0);
          iv.push_back(lxh[q]);
        }
      }
      for (int64_t q = up[s]; q < up[s + 1]; ++q)
        if (ui[q] >= B.s0 + B.m) {
          bi.push_back(ui[q]);
          bv.push_back(ux[q]);
        }
      ep[t + 1] = (int64_t)ei.size();
      bp[t + 1] = (int64_t)bi.size();
      ip[t + 1] = (int64_t)ii.size();
    }
    B.nfe = (int64_t)ei.size();
    B.nbe = (int64_t)bi.size();
    D.sweep_entries += B.nfe + B.nbe;
    if (g_opt.verbose)
      std::fprintf(stderr, "block rows %d..%d (%d, %s): external entries %lld forward, %lld backward\n", B.s0,
                   B.s0 + B.m - 1, B.m, gr.dense ? "explicit inverse" : "gather only", (long long)B.nfe,
                   (long long)B.nbe);
    up_(B.ep, ep);
    up_(B.ei, ei);
    up_(B.ev, ev);
    up_(B.bp, bp);
    up_(B.bi, bi);
    up_(B.bv, bv);
    if (gr.dense) {
      std::vector<S> tf, tb;
      tail_inverse<H, S>(B.m, ip, ii, iv, tf, tb, nth, [](const H& v) { return StoreOf<S>::f(v); });
      B.nt = (B.m + kTile - 1) / kTile;
      B.tcl = tile_cluster<S>();
      const std::vector<int> itf = make_cluster_items(B.nt, true, B.tcl),
                             itb = make_cluster_items(B.nt, false, B.tcl);
      up_(B.tf, tf);
      up_(B.tb, tb);
      up_(B.itf, itf);
      up_(B.itb, itb);
      B.nitf = (int)(itf.size() / 4);
      B.nitb = (int)(itb.size() / 4);
      max_items = std::max(max_items, (size_t)B.m);
      D.tile_bytes += 2.0 * (double)tf.size() * sizeof(S);
    }
    CK(cudaStreamSynchronize(st));  // the host vectors of this block are released next
    D.blocks.push_back(B);
  }
  if (max_items > 0) D.xb = (A*)alloc(sizeof(A) * max_items);
  D.y = (A*)alloc(sizeof(A) * std::max(1, n));
  if (graph_io) {  // the input and output vectors of the captured application graph
    D.rhs_in = alloc(sizeof(zc) * std::max(1, n));
    D.sol_out = alloc(sizeof(zc) * std::max(1, n));
  }
  k::ildl_plan(D, lp, up, brs);
  k::ildl_plan_bwd0(D, up, brs);
  CK(cudaStreamSynchronize(st));
  if (g_opt.verbose || g_opt.factor_verbose) {
    int dense_b = 0;
    for (const auto& B : D.blocks) dense_b += B.nt > 0;
    std::fprintf(stderr,
                 "factor upload: n %d, L %lld, forward levels %d (bulk %d), sweep kernels %zu + %zu, blocks %zu "
                 "(%d dense, %d rows)\n",
                 n, (long long)D.nnz_l, nfl, Lt, D.fseg.size() / 3, D.bseg.size() / 3, D.blocks.size(), dense_b,
                 m_tail);
  }
}

// A factor with coupling blocks: every level becomes a sub-factor (its rows in
// elimination order, identity permutation, the level's own L and D), F and
// F^H are stored as CSR over elimination steps, plus the work vectors of the
// composed application (k::ildl_apply).
template <class S, class H, class Alloc>
void upload_coupled(const IldlcFactor<H>& F, DevFactor<S>& D, cudaStream_t st, Alloc alloc, bool graph_io) {
  const int n = F.n;
  const int nl = (int)F.level_start.size() - 1;
  D.n = n;
  D.coupled = 1;
  D.lstart = F.level_start;
  D.lev.resize(nl);
  for (int l = 0; l < nl; ++l) {
    const int a = F.level_start[l], e = F.level_start[l + 1], m = e - a;
    IldlcFactor<H> sub;
    sub.n = m;
    sub.perm.resize(m);
    for (int i = 0; i < m; ++i) sub.perm[i] = i;
    sub.lp.assign(m + 1, 0);
    for (int p = a; p < e; ++p) sub.lp[p - a + 1] = sub.lp[p - a] + (F.lp[p + 1] - F.lp[p]);
    sub.li.resize(sub.lp[m]);
    sub.lx.resize(sub.lp[m]);
    for (int p = a; p < e; ++p)
      for (int64_t q = F.lp[p], o = sub.lp[p - a]; q < F.lp[p + 1]; ++q, ++o) {
        if (F.li[q] < a) throw std::runtime_error("coupled factor: an L entry crosses a level");
        sub.li[o] = F.li[q] - a;
        sub.lx[o] = F.lx[q];
      }
    sub.blk.assign(F.blk.begin() + a, F.blk.begin() + e);
    sub.dinv.assign(F.dinv.begin() + a, F.dinv.begin() + e);
    sub.doff.assign(F.doff.begin() + a, F.doff.begin() + e);
    sub.ainv.assign(F.ainv.begin() + a, F.ainv.begin() + e);
    sub.aoff.assign(F.aoff.begin() + a, F.aoff.begin() + e);
    sub.level_start = {0, m};
    upload_factor(sub, D.lev[l], st, alloc, false);
    // each level below the last is solved twice per application
    const int mult = l + 1 < nl ? 2 : 1;
    D.nnz_l += D.lev[l].nnz_l;
    D.sweep_entries += mult * D.lev[l].sweep_entries;
    D.tile_bytes += mult * D.lev[l].tile_bytes;
  }
  // F (rows: steps of each level's pivots, one CSR over all steps) and, per
  // level l, F_l^H over the steps after the level: rows e_l..n-1 with their
  // entries in the level's columns, row pointers of all levels in one array
  std::vector<S> fpx(F.fi.size());
  for (size_t q = 0; q < F.fi.size(); ++q) fpx[q] = StoreOf<S>::f(F.fx[q]);
  std::vector<int64_t> fhp;
  std::vector<int> fhi(F.fi.size());
  std::vector<S> fhx(F.fi.size());
  D.fh_row0.assign(std::max(0, nl - 1), 0);
  D.fp_lanes.assign(nl, 8);
  D.fh_lanes.assign(nl, 8);
  int64_t base = 0;  // entries of the earlier levels' blocks
  for (int l = 0; l + 1 < nl; ++l) {
    const int a = F.level_start[l], e = F.level_start[l + 1], m = n - e;
    D.fh_row0[l] = (int64_t)fhp.size();
    std::vector<int64_t> rp(m + 1, 0);
    for (int p = a; p < e; ++p)
      for (int64_t q = F.fp[p]; q < F.fp[p + 1]; ++q) rp[F.fi[q] - e + 1]++;
    for (int t = 0; t < m; ++t) rp[t + 1] += rp[t];
    std::vector<int64_t> w(rp.begin(), rp.end() - 1);
    for (int p = a; p < e; ++p)
      for (int64_t q = F.fp[p]; q < F.fp[p + 1]; ++q) {
        const int64_t o = base + w[F.fi[q] - e]++;
        fhi[o] = p;
        fhx[o] = StoreOf<S>::f(jdd::cj(F.fx[q]));
      }
    for (auto& v : rp) v += base;
    fhp.insert(fhp.end(), rp.begin(), rp.end());
    base = rp[m];
    D.fp_lanes[l] = k::lanes_per_row((double)(F.fp[e] - F.fp[a]) / std::max(1, e - a));
    D.fh_lanes[l] = k::lanes_per_row((double)(rp[m] - rp[0]) / std::max(1, m));
  }
  if (base != (int64_t)F.fi.size()) throw std::runtime_error("coupled factor: F entries outside their levels");
  D.nnz_f = (int64_t)F.fi.size();
  auto up_ = [&](auto*& dst, const auto& src) {
    using E = typename std::remove_reference<decltype(src)>::type::value_type;
    dst = (std::remove_reference_t<decltype(dst)>)alloc(sizeof(E) * std::max<size_t>(1, src.size()));
    if (!src.empty()) CK(cudaMemcpyAsync(dst, src.data(), sizeof(E) * src.size(), cudaMemcpyHostToDevice, st));
  };
  up_(D.perm, F.perm);
  up_(D.fpp, F.fp);
  up_(D.fpi, F.fi);
  up_(D.fpx, fpx);
  up_(D.fhp, fhp);
  up_(D.fhi, fhi);
  up_(D.fhx, fhx);
  D.cy = alloc(sizeof(H) * std::max(1, n));
  D.cyb = alloc(sizeof(H) * std::max(1, n));
  D.ct = alloc(sizeof(H) * std::max(1, n));
  if (graph_io) {
    D.rhs_in = alloc(sizeof(zc) * std::max(1, n));
    D.sol_out = alloc(sizeof(zc) * std::max(1, n));
  }
  CK(cudaStreamSynchronize(st));  // the host arrays are released next
}

template <class T> struct LowOf { using type = float; using bf = __nv_bfloat16; };
template <> struct LowOf<zc> { using type = cc; using bf = bc; };

// ------------------------------------------------------- global state ----

template <class T> struct Global {
  using H = typename HostOf<T>::type;
  using L = typename LowOf<T>::type;
  using B = typename LowOf<T>::bf;
  double timefact = -1, shift0 = 0, droptol0 = 0, diagmin = 0, shiftmax = 0, memrequested = 0, memused = 0,
         condest0 = 5;
  const double slightlyless = 0.8, toldiv = 2.0;
  int factdgl = 0, factspd = 0, prvdr = 0;
  int precision = 0;  // 0: factor in T, 1: single (ICNTL(5)=1), 2: bfloat16 storage
  bool reenterfirsttime = false;
  JdState sh;
  Workspace<T> W;
  IldlcFactor<H> F;        // host factor (kept for re-upload / information)
  DevFactor<T> Fd;         // device factor, full precision
  DevFactor<L> Fs;         // device factor, single precision
  DevFactor<B> Fb;         // device factor, bfloat16 storage
  double* ddiag = nullptr; // diagonal preconditioner on the device
  SellMatrix<T> A, Bm;     // built-in matvec operands
  bool resident = false;   // A (and B) prepared on the device by the caller
  int nfactor = 0;
  double t_factor = 0, t_upload = 0;
  long n_precond = 0, n_matvec = 0;
  int last_levels = 0, last_fdepth = 0, last_bdepth = 0;
  int factor_threads = 0;  // host threads of the factorisation (0: all, at most 16)
  void cleanup1() {
    factdgl = 0;
    F = IldlcFactor<H>();
    free_factor(Fd);
    free_factor(Fs);
    free_factor(Fb);
    if (ddiag) { cudaFree(ddiag); ddiag = nullptr; }
  }
  void release() {
    cleanup1();
    free_sell(A);
    free_sell(Bm);
    resident = false;
    W.release();
  }
};
// The solver state of an arithmetic: one per process (the reference's COMMON
// blocks) unless the calling thread installed its own (batch workers).
template <class T> Global<T>*& thread_global() {
  static thread_local Global<T>* p = nullptr;
  return p;
}
template <class T> Global<T>& G() {
  static Global<T> g;
  Global<T>* p = thread_global<T>();
  return p ? *p : g;
}

template <class H> static void diag_first(int n, int* ia, int* ja, H* a) {
  for (int i = 0; i < n; ++i)
    for (int j = ia[i] - 1; j < ia[i + 1] - 1; ++j)
      if (ja[j] - 1 == i) {
        int l = ia[i] - 1;
        std::swap(ja[j], ja[l]);
        std::swap(a[j], a[l]);
      }
}

template <class H> static double savediag_shift(int n, const int* ia, const int* ja, const H* a) {
  std::vector<double> disc(n, 0.0), dg(n, 0.0);
  int ki = 0;
  double ti = 0;
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j) {
      int k = ja[j - 1] - 1;
      if (k == i) {
        dg[i] = hre(a[j - 1]);
        if (i == 0) ti = hre(a[j - 1]);
        else {
          if (hre(a[j - 1]) < ti) ti = hre(a[j - 1]);
          ki = i;
        }
      } else {
        double v = habs(a[j - 1]);
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

template <class H>
static double savediag_shift_gep(int n, const int* ia, const int* ja, const H* a, const int* ib, const int* jb,
                                 const H* b) {
  std::vector<double> disc(n, 0.0), dg(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = ib[i]; j < ib[i + 1]; ++j)
      if (jb[j - 1] - 1 == i) dg[i] = hre(b[j - 1]);
  for (int i = 0; i < n; ++i)
    for (int j = ib[i]; j < ib[i + 1]; ++j) {
      int k = jb[j - 1] - 1;
      if (k != i) {
        double val = std::sqrt(dg[i] / dg[k]);
        dg[i] += habs(b[j - 1]) * val;
        dg[k] += habs(b[j - 1]) / val;
      }
    }
  for (int i = 0; i < n; ++i) dg[i] = 1 / std::sqrt(dg[i]);
  int ki = 0;
  double ti = 0;
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j) {
      int k = ja[j - 1] - 1;
      if (k == i) {
        double val = dg[i] * hre(a[j - 1]) * dg[k];
        if (i == 0) ti = val;
        else if (val < ti) { ti = val; ki = i; }
      } else {
        double val = dg[i] * habs(a[j - 1]) * dg[k];
        disc[i] += val;
        disc[k] += val;
      }
    }
  for (int i = 0; i < n; ++i)
    for (int j = ia[i]; j < ia[i + 1]; ++j)
      if (ja[j - 1] - 1 == i) dg[i] = dg[i] * hre(a[j - 1]) * dg[i];
  double val = ti - disc[ki];
  for (int i = 0; i < n; ++i) {
    double tmp = dg[i] - disc[i];
    if (tmp < val && dg[i] - ti < disc[ki]) val = tmp;
  }
  return val;
}

struct PrecondFailure {};
struct RevcomCancelled {};

struct Printer {
  int pr = 0;  // 0 errors only, 1 standard, 2 expert
  void set(int iprint) { pr = iprint == 0 ? 0 : (iprint < 0 ? 2 : 1); }
};

// DGLPRECSETUP (a holds the n diagonal entries)
template <class T>
void dglprecsetup(Global<T>& g, const typename HostOf<T>::type* a, int n, int isearch, double shift, double& shift0) {
  std::vector<double> d(n, 0.0);
  double dmin = hre(a[0]), ta = dmin;
  for (int i = 1; i < n; ++i) {
    dmin = std::min(dmin, hre(a[i]));
    ta = std::max(ta, hre(a[i]));
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
    for (int i = 0; i < n; ++i) d[i] = 1.0 / (hre(a[i]) - shift0);
  } else {
    g.factspd = 0;
    del = 1.0 / del;
    for (int i = 0; i < n; ++i) {
      double t = hre(a[i]) - shift0;
      t = (t > 0) ? std::max(t, del) : std::min(t, -del);
      d[i] = 1.0 / t;
    }
  }
  if (g.ddiag) cudaFree(g.ddiag);
  CK(cudaMalloc(&g.ddiag, sizeof(double) * n));
  CK(cudaMemcpy(g.ddiag, d.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  g.factdgl = 1;
}

// PJDINIT: returns ierr
template <class T>
int pjdinit(Global<T>& g, Printer& P, int n, typename HostOf<T>::type* a, int* ja, int* ia,
            const typename HostOf<T>::type* b, const int* jb, const int* ib, double sigma, int isearch, double& SHIFT,
            double& DROPTOL, double& MEM, const int* icntl, bool gep) {
  using H = typename HostOf<T>::type;
  if (g.factdgl != 0) g.cleanup1();
  if (ja[0] < 0) {
    if (isearch >= 2) g.shift0 = sigma;
    double s0 = g.shift0;
    dglprecsetup(g, a, n, isearch, SHIFT, s0);
    g.shift0 = s0;
    if (P.pr >= 1)
      std::printf("\n- Setting up a new diagonal preconditioner -------------\nused shift:%12.4E\n"
                  "--------------------------------------------------------\n", g.shift0);
    return 0;
  }
  if (DROPTOL < 0) DROPTOL = 1e-2;
  double condest = (g.timefact > 0) ? g.condest0 : (icntl[3] <= 0 ? 5.0 : (double)icntl[3]);
  if (MEM <= 0) MEM = 10.0;
  int newsh = 0;
  for (;;) {
    double tic = wall();
    if (P.pr >= 1) std::printf("\n- Setting up a new ILU preconditioner ------------------\n");
    g.diagmin = 0;
    for (int i = 0; i < n; ++i) {
      double val = 0;
      for (int j = ia[i] - 1; j < ia[i + 1] - 1; ++j)
        if (ja[j] - 1 == i) val = hre(a[j]);
      g.diagmin = (i == 0) ? val : std::min(val, g.diagmin);
    }
    g.shift0 = gep ? savediag_shift_gep(n, ia, ja, a, ib, jb, b) : savediag_shift(n, ia, ja, a);
    if (isearch >= 2) g.shift0 = sigma;
    int ggsh = 0;
    if (isearch == 1 && SHIFT < g.diagmin) g.shift0 = SHIFT;
    else ggsh = 1;
    if (isearch <= 0 && newsh == 1) g.shift0 = SHIFT;
    if (newsh != 1 && g.timefact <= 0) g.shiftmax = g.diagmin;
    g.memrequested = MEM;
    const int recompilu = (icntl[1] == 0 || icntl[1] == -2) ? 1 : -1;
    const double nposeig = (icntl[2] <= 0) ? 0.01 : 0.0;
    IldlcParams prm;
    prm.droptol = DROPTOL;
    prm.condest = condest;
    prm.mem = MEM;
    factor_options(prm, n, isearch);
    prm.threads = g.factor_threads;
    double tf0 = wall();
    int ierr = ildlc_factor<H>(n, ia, ja, a, g.shift0, gep ? ib : nullptr, gep ? jb : nullptr, gep ? b : nullptr,
                               prm, g.F);
    g.t_factor += wall() - tf0;
    g.nfactor++;
    g.memused = (ierr == 0) ? g.F.fill() + 0.05 : MEM;
    diag_first(n, ia, ja, a);
    if (ierr == -3 || ierr == -2) {
      if (!(recompilu == -1 || g.prvdr == -1)) {
        g.prvdr = 1;
        DROPTOL = DROPTOL * 2 * g.toldiv;
        std::printf("Not enough memory: factorization will be restarted with larger DROPTOL %8.1E\n", DROPTOL);
        g.cleanup1();
        continue;
      }
      std::printf("Not enough memory: factorization should be restarted with larger DROPTOL\n");
    } else if (ierr == -5 || ierr == -6 || ierr > 0) {
      if (!(recompilu == -1 || g.prvdr == 1) && g.memused < g.slightlyless * g.memrequested) {
        if (g.memused < (3 * g.slightlyless - 2) * g.memrequested) DROPTOL /= 4 * g.toldiv;
        else if (g.memused < (2 * g.slightlyless - 1) * g.memrequested) DROPTOL /= 2 * g.toldiv;
        else DROPTOL /= g.toldiv;
        DROPTOL = std::max(DROPTOL, 1.01 * std::sqrt(DBL_EPSILON * 0.5));
        g.prvdr = -1;
        std::printf("zero pivot encountered: factorization will be restarted with smaller DROPTOL %8.1E\n", DROPTOL);
        g.cleanup1();
        continue;
      }
      std::printf("reduce DROPTOL and increase MEM! (zero pivot encountered)\n");
    } else if (ierr == -1) {
      std::printf("Error. input matrix may be wrong.\n");
    }
    if (ierr != 0) {
      g.cleanup1();
      return ierr;
    }
    double totaltime = wall() - tic;
    if (P.pr >= 1)
      std::printf(" fill-in factor:%10.2f (=nnz(LU)/nnz(A))\n   used droptol: %13.5E\n     used shift: %13.5E\n",
                  g.F.fill(), DROPTOL, g.shift0);
    if (P.pr >= 1) std::printf("   ILU computed:%10.2f[sec]\n", totaltime);
    g.factspd = 0;
    if (isearch <= 1) {
      g.factspd = g.F.nneg;
      if (g.factspd > 0) {
        if (!(recompilu == -1 || g.factspd <= n * nposeig)) {
          g.shiftmax = std::min(g.shift0, g.shiftmax);
          SHIFT = 2 * SHIFT - g.diagmin;
          newsh = 1;
          g.prvdr = std::min(g.prvdr, 0);
          std::printf("Too many neg. diagonal entries:\nfactorization will be restarted with smaller shift %12.4E\n", SHIFT);
          g.cleanup1();
          continue;
        }
        if (P.pr >= 1) std::printf("ILU-> pos. def.:%10d negative diag. entries changed to positive\n", g.factspd);
      } else if (isearch <= 0 || newsh == 1 || ggsh == 1) {
        g.factspd = -1;
      }
    }
    // upload the factor in the requested precision
    double tu = wall();
    if (g.precision == 1) upload_factor(g.F, g.Fs, g.W.st);
    else if (g.precision == 2) upload_factor(g.F, g.Fb, g.W.st);
    else upload_factor(g.F, g.Fd, g.W.st);
    g.t_upload += wall() - tu;
    {
      std::vector<int> fp, fr, bp, br;
      ildlc_levels(g.F, fp, fr, bp, br);
      g.last_levels = (int)g.F.level_start.size() - 1;
      g.last_fdepth = (int)fp.size() - 1;
      g.last_bdepth = (int)bp.size() - 1;
    }
    g.timefact = std::max(totaltime, 1e-2);
    g.factdgl = -1;
    g.droptol0 = DROPTOL;
    g.condest0 = condest;
    if (P.pr >= 1) std::printf("--------------------------------------------------------\n");
    return 0;
  }
}

// The preconditioner-aware driver (PJDRVCOM).  user_mv: reverse-communication
// matvec requests; nullptr means the built-in device SpMV.
template <class T> struct PjdRun {
  using H = typename HostOf<T>::type;
  Global<T>& g;
  Printer P;
  int n;
  H *a, *b;
  int *ia, *ja, *ib, *jb;
  bool gep;
  int* NEIGp;
  double* EIGS;
  double* GAPp;
  int NW = 0, ISEARCH = 0;
  int* ICNTL;
  double SIGMA = 0, TOL = 0;
  double *SHIFT, *DROPTOL, *MEM;
  double tic = 0, rprev = 1;
  std::function<void(int, long, long, long)> user_mv;
  DevJd<T> jd;
  explicit PjdRun(Global<T>& gg) : g(gg) {}

  void builtin_mv(int which, long x, long y, long by) {
    g.n_matvec++;
    if (which == 1 || which == 3) k::spmv<T>(g.A, jd.D(x), jd.D(y), g.W.st);
    if ((which == 1 || which == 4) && gep) k::spmv<T>(g.Bm, jd.D(x), jd.D(by), g.W.st);
  }
  void builtin_mv_shift(long x, long y, typename HostOf<T>::type a) {
    g.n_matvec++;
    k::spmv_shift<T>(g.A, todev(a), jd.D(x), jd.D(y), g.W.st);
  }
  void precond(long rhs, long sol);
};

template <class T> void PjdRun<T>::precond(long rhs, long sol) {
  JdState& S = g.sh;
  const double EPSMACH = DBL_EPSILON * 0.5;
  const int NEIG = *NEIGp;
  double& SH = *SHIFT;
  double& DT = *DROPTOL;
  bool reinit = false;
  int factspd0 = 0;
  double toc = wall();
  auto E = [&](int i) { return EIGS[i - 1]; };
  if (g.factdgl > 0 && !S.flagcg && ISEARCH <= 1 && (ICNTL[1] == 0 || ICNTL[1] == -2) && ICNTL[0] != 2) {
    double tent;
    if (NEIG >= 1) { tent = E(NW); factspd0 = -1; }
    else {
      tent = S.shift1 - S.rcurr;
      factspd0 = -1;
      if (10 * S.rcurr >= g.diagmin - tent && S.shift1 > g.shift0) factspd0 = g.factspd;
    }
    if (g.diagmin > tent && factspd0 < 0 && 10 * std::fabs(g.shift0 - tent) >= (g.diagmin - g.shift0)) {
      SH = tent;
      reinit = true;
    }
  }
  if (g.factdgl < 0 && !S.flagcg && (ICNTL[1] == 0 || ICNTL[1] == -2) && ICNTL[0] != 2 &&
      S.rcum - rprev <= 6 * std::log(S.rinit / TOL)) {
    CK(cudaStreamSynchronize(g.W.st));
    toc = wall();
    double tmsol = toc - tic, time0, time1;
    if (tmsol < 1e-1) tmsol = 0;
    if (S.rcum > rprev) {
      time1 = tmsol * std::log(S.rinit / TOL) / (S.rcum - rprev);
      time0 = tmsol * std::log(S.rcurr / TOL) / (S.rcum - rprev);
    } else {
      time1 = 4 * g.timefact;
      time0 = 6 * g.timefact;
    }
    if (2 * g.timefact < time1 && 4 * g.timefact < time0 + (NW - NEIG - 1) * time1) {
      if (g.factspd < 0) {
        double tent, delta;
        if (NEIG >= 1) {
          delta = (NEIG > 1) ? std::fabs(E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*GAPp, 0.0);
          tent = std::min(2 * g.shiftmax - E(NW), E(NW) - delta);
        } else {
          tent = std::min(2 * g.shiftmax - S.shift1, S.shift1 - S.rcurr - std::max(*GAPp, 0.0));
          if (2 * S.rcurr >= g.diagmin - tent) factspd0 = g.factspd;
        }
        if ((factspd0 == 0 || 4 * g.timefact < time0) && g.diagmin > tent &&
            2 * (tent - g.shift0) >= (g.diagmin - g.shift0)) {
          SH = tent;
          rprev = S.rcum;
          reinit = true;
        }
      }
      if (factspd0 >= 0 && !reinit && g.memused < g.slightlyless * g.memrequested && g.prvdr <= 0 &&
          DT >= std::sqrt(EPSMACH)) {
        if (ICNTL[1] != -2) g.reenterfirsttime = false;
        double DT0 = DT;
        if (!g.reenterfirsttime) {
          if (g.memused < (3 * g.slightlyless - 2) * g.memrequested) DT /= 4 * g.toldiv;
          else if (g.memused < (2 * g.slightlyless - 1) * g.memrequested) DT /= 2 * g.toldiv;
          else DT /= g.toldiv;
          DT = std::max(DT, 1.01 * std::sqrt(EPSMACH));
        }
        rprev = S.rcum;
        reinit = true;
        if (DT == 1.01 * std::sqrt(EPSMACH) && DT0 == DT && !g.reenterfirsttime) reinit = false;
        g.reenterfirsttime = false;
        SH = g.shift0;
        if (g.factspd > 0) {
          if (NEIG >= 1) {
            double delta = (NEIG > 1) ? (E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*GAPp, 0.0);
            SH = std::min(std::min(2 * g.shift0 - E(NW), E(NW) - delta), g.shiftmax);
          } else if (g.shift0 > S.shift1) {
            SH = std::min(S.shift1, g.shiftmax);
          }
        }
      } else if (g.factspd > 0) {
        if (NEIG >= 1) {
          if (g.shift0 > E(NW)) {
            double delta = (NEIG > 1) ? (E(NW) - E(NW - NEIG + 1)) / (NEIG - 1) : std::max(*GAPp, 0.0);
            SH = std::min(E(NW) - delta, g.shiftmax);
            rprev = S.rcum;
            reinit = true;
          }
        } else if (g.shift0 > S.shift1 && 2 * (g.shift0 - S.shift1) >= (g.diagmin - g.shift0)) {
          SH = std::min(S.shift1, g.shiftmax);
          rprev = S.rcum;
          reinit = true;
        }
      }
    }
  }
  if (reinit) {
    int ierr = pjdinit(g, P, n, a, ja, ia, b, jb, ib, SIGMA, std::max(ISEARCH, 1), SH, DT, *MEM, ICNTL, gep);
    if (ierr != 0) {
      g.factdgl = 1;
      throw PrecondFailure();
    }
    double t = wall();
    S.timeilu += std::max(t - toc, 0.0);
    tic = t;
    if (factspd0 < 0 && g.factspd <= 0) g.factspd = factspd0;
  }
  g.n_precond++;
  if (g.factdgl > 0) {
    k::diagsolve<T>(n, g.ddiag, jd.D(rhs), jd.D(sol), g.W.st);
  } else {
    const bool spd = ISEARCH <= 1;
    if (g.precision == 1) k::ildl_apply_graph<T, typename Global<T>::L>(g.Fs, spd, jd.D(rhs), jd.D(sol), g.W.st);
    else if (g.precision == 2) k::ildl_apply_graph<T, typename Global<T>::B>(g.Fb, spd, jd.D(rhs), jd.D(sol), g.W.st);
    else k::ildl_apply_graph<T, T>(g.Fd, spd, jd.D(rhs), jd.D(sol), g.W.st);
  }
}

template <class T> static void print_table(Printer& P, const double* EIGS, const double* RES, int NEIG, int ITER,
                                           double GAP, int INFO, double tsolve) {
  if (P.pr < 1) return;
  std::printf("\n            Eigenvalue     Res. norm    Error est.   No(Cluster)\n");
  for (int i = 0; i < NEIG; ++i) std::printf("%22.13E%14.1E\n", EIGS[i], RES[i]);
  std::printf("\n  Number of MATVEC needed:%7d ;  Estimated gap:%9.2E ;  INFO:%3d\n\n", ITER, GAP, INFO);
  std::printf("CPU time for eigenvalue computation:%10.2f[sec]\n", tsolve);
}

// Runs PJDRVCOM (built-in or user matvec).  All pointers are the caller's.
template <class T>
void pjd_drive(int n, typename HostOf<T>::type* a, int* ja, int* ia, typename HostOf<T>::type* b, int* jb, int* ib,
               double* EIGS, double* RES, typename HostOf<T>::type* X, int LX, int* NEIG, double SIGMA, int ISEARCH,
               int NINIT, int MADSPACE, int* ITER, double TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL,
               int IPRINT, int* INFO, double* GAP, bool gep, std::function<void(int, long, long, long)> user_mv,
               DevJd<T>** jd_out = nullptr) {
  using H = typename HostOf<T>::type;
  Global<T>& g = G<T>();
  JdState& S = g.sh;
  PjdRun<T> R(g);
  R.P.set(IPRINT);
  g.precision = ICNTL[4] == 1 ? 1 : (ICNTL[4] == 2 ? 2 : 0);
  const double t0 = wall();
  if (R.P.pr >= 1) {
    std::printf("\n**ENTERING PJDREVCOM************************************\n\n");
    if (ISEARCH <= 1) std::printf("Computing the smallest eigenvalue(s)\n------------------------------------\n");
    else std::printf("Computing the eigenvalue(s) closest to %12.5E\n---------------------------------------------------\n", SIGMA);
  }
  long lxl = LX;
  g.W.ensure(n, lxl);
  int ierr = 0;
  if ((ICNTL[1] != -1 && ICNTL[1] != -2) || g.factdgl == 0) {
    g.prvdr = 0;
    g.timefact = -1;
    g.cleanup1();
    ierr = pjdinit(g, R.P, n, a, ja, ia, b, jb, ib, SIGMA, ISEARCH, *SHIFT, *DROPTOL, *MEM, ICNTL, gep);
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
          if (ja[j] - 1 == i) val = hre(a[j]);
        g.diagmin = (i == 0) ? val : std::min(val, g.diagmin);
      }
      if (!gep) g.shift0 = savediag_shift(n, ia, ja, a);
      if (ISEARCH >= 2) g.shift0 = SIGMA;
      if (ISEARCH == 1 && *SHIFT < g.diagmin) g.shift0 = *SHIFT;
      diag_first(n, ia, ja, a);
      S.timeilu = 0;
      // a kept factor reused in another storage precision (ICNTL(5) changed
      // between the calls): upload the host factor in that precision once
      if (g.F.n == n) {
        double tu = wall();
        if (g.precision == 1 && g.Fs.n != n) upload_factor(g.F, g.Fs, g.W.st);
        else if (g.precision == 2 && g.Fb.n != n) upload_factor(g.F, g.Fb, g.W.st);
        else if (g.precision == 0 && g.Fd.n != n) upload_factor(g.F, g.Fd, g.W.st);
        g.t_upload += wall() - tu;
      }
    }
  }
  if (ierr != 0) {
    *INFO = -54321;
    return;
  }
  const double t1 = wall();
  // operands of the built-in matvec
  if (!user_mv && !g.resident) {
    if (ja[0] < 0) throw std::runtime_error("diagonal preconditioning needs the reverse-communication matvec");
    build_sell<T>(n, ia, ja, a, g.A, g.W.st);
    if (gep) build_sell<T>(n, ib, jb, b, g.Bm, g.W.st);
  }
  // initial guesses
  if (NINIT > 0)
    CK(cudaMemcpyAsync(g.W.dX, X, sizeof(T) * (size_t)n * NINIT, cudaMemcpyHostToDevice, g.W.st));
  R.n = n; R.a = a; R.b = b; R.ia = ia; R.ja = ja; R.ib = ib; R.jb = jb;
  R.gep = gep;
  R.NEIGp = NEIG;
  R.EIGS = EIGS;
  R.GAPp = GAP;
  R.NW = *NEIG;
  R.ISEARCH = ISEARCH;
  R.ICNTL = ICNTL;
  R.SIGMA = SIGMA;
  R.TOL = TOL;
  R.SHIFT = SHIFT;
  R.DROPTOL = DROPTOL;
  R.MEM = MEM;
  R.tic = wall();
  R.rprev = 1.0;
  R.user_mv = user_mv;
  DevJd<T>& jd = R.jd;
  jd.W = &g.W;
  jd.sh = &S;
  jd.hX = X;
  if (user_mv) jd.matvec = user_mv;
  else jd.matvec = [&R](int w, long x, long y, long by) { R.builtin_mv(w, x, y, by); };
  jd.precond = [&R](long r, long s) { R.precond(r, s); };
  jd.device_ops = !user_mv && g_opt.fuse_inner != 0;
  if (jd.device_ops && !gep)
    jd.matvec_shift = [&R](long x, long y, typename HostOf<T>::type a) { R.builtin_mv_shift(x, y, a); };
  if (R.P.pr >= 2)
    jd.on_step = [](int conv, int step, int k, double th, double v) {
      if (conv) std::printf("Step:%4d(%3d) ;  #MV:%7d ;  Rayl. quot.:%12.5E * converged\n\n", step, k, (int)v, th);
      else std::printf("Step:%4d(%3d) ;  Rayl. quot.:%12.5E ;  Res. norm:%8.1E\n", step, k, th, v);
    };
  if (jd_out) *jd_out = &jd;
  try {
    jd.run(n, EIGS, RES, LX, *NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, *ITER, TOL, *INFO, *GAP, gep);
  } catch (PrecondFailure&) {
    *INFO = -54321;
    return;
  }
  // eigenvectors back to the caller (kept on the device in resident mode)
  int nv = std::max(*NEIG, 0) + ((*INFO > 0) ? 1 : 0);
  if (g.resident) nv = 0;
  nv = std::min(nv, std::max(1, R.NW));
  if (nv > 0) CK(cudaMemcpyAsync(X, g.W.dX, sizeof(T) * (size_t)n * nv, cudaMemcpyDeviceToHost, g.W.st));
  if (gep && nv > 0) {
    long BX = (long)R.NW * n + (long)std::min(MADSPACE, n) * n * 2;
    CK(cudaMemcpyAsync(X + BX, g.W.dX + BX, sizeof(T) * (size_t)n * nv, cudaMemcpyDeviceToHost, g.W.st));
  }
  CK(cudaStreamSynchronize(g.W.st));
  const double t2 = wall();
  print_table<T>(R.P, EIGS, RES, *NEIG, *ITER, *GAP, *INFO, t2 - t1);
  if (R.P.pr >= 1)
    std::printf("       CPU time for preconditioning:%10.2f[sec]\n                     Total CPU time:%10.2f[sec]\n",
                S.timeilu + (t1 - t0), t2 - t0);
  // suggested SHIFT / DROPTOL for a restart
  *SHIFT = g.shift0;
  if (g.factdgl >= 0) {
    *SHIFT = EIGS[0];
  } else if (g.factspd != 0 || ISEARCH <= 0) {
    int ne = *NEIG;
    double delta = (ne > 1) ? (EIGS[ne - 1] - EIGS[0]) / (ne - 1) : std::max(*GAP, 0.0);
    if (g.factspd > 0) {
      *SHIFT = std::min(*SHIFT, g.shiftmax);
      *SHIFT = std::min(2 * *SHIFT - EIGS[0], EIGS[0] - delta);
    } else {
      *SHIFT = std::min(2 * g.shiftmax - EIGS[0], EIGS[0] - delta);
      if (g.shift0 < EIGS[0]) *SHIFT = std::max(*SHIFT, g.shift0);
    }
  }
  if (R.P.pr >= 1 && ISEARCH <= 1) std::printf(" (Suggested SHIFT   if restart needed:%9.2E)\n", *SHIFT);
  if (R.P.pr >= 1 && g.factdgl <= 0) std::printf(" (Suggested DROPTOL if restart needed:%9.2E)\n", *DROPTOL);
  if (R.P.pr >= 1) std::printf("\n**LEAVING PJDREVCOM*************************************\n\n");
}

// JDREVCOM: user matvec and user preconditioner
template <class T>
void jd_drive(int n, double* EIGS, double* RES, typename HostOf<T>::type* X, int LX, int* NEIG, double SIGMA,
              int ISEARCH, int NINIT, int MADSPACE, int* ITER, double TOL, int IPRINT, int* INFO, double* GAP,
              bool gep, std::function<void(int, long, long, long)> user_mv, std::function<void(long, long)> user_pc) {
  Global<T>& g = G<T>();
  g.W.ensure(n, LX);
  if (NINIT > 0)
    CK(cudaMemcpyAsync(g.W.dX, X, sizeof(T) * (size_t)n * NINIT, cudaMemcpyHostToDevice, g.W.st));
  DevJd<T> jd;
  jd.W = &g.W;
  jd.sh = &g.sh;
  jd.hX = X;
  jd.matvec = user_mv;
  jd.precond = user_pc;
  int nw = *NEIG;
  jd.run(n, EIGS, RES, LX, *NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, *ITER, TOL, *INFO, *GAP, gep);
  int nv = std::min(std::max(*NEIG, 0) + ((*INFO > 0) ? 1 : 0), std::max(1, nw));
  CK(cudaMemcpyAsync(X, g.W.dX, sizeof(T) * (size_t)n * nv, cudaMemcpyDeviceToHost, g.W.st));
  CK(cudaStreamSynchronize(g.W.st));
  Printer P;
  P.set(IPRINT);
  print_table<T>(P, EIGS, RES, *NEIG, *ITER, *GAP, *INFO, 0.0);
}

// ------------------------------------------------ reverse communication ----
struct Revcom {
  std::thread th;
  std::mutex m;
  std::condition_variable cv;
  enum State { IDLE, RUNNING, REQUEST, DONE } state = IDLE;
  int ijob = 0, ndx1 = 0, ndx2 = 0, ndx3 = 0;
  bool cancel = false;
  bool device = false;  // requests served on the device copy of X
  std::string error;
  // worker side: post a request and wait for the caller to serve it
  void request(int job, long x1, long x2, long x3) {
    std::unique_lock<std::mutex> lk(m);
    ijob = job;
    ndx1 = (int)x1 + 1;
    ndx2 = (int)x2 + 1;
    ndx3 = (int)x3 + 1;
    state = REQUEST;
    cv.notify_all();
    cv.wait(lk, [&] { return state == RUNNING || cancel; });
    if (cancel) throw RevcomCancelled();
  }
  // caller side
  void start(std::function<void()> body) {
    finish_old();
    cancel = false;
    error.clear();
    state = RUNNING;
    th = std::thread([this, body] {
      try {
        body();
      } catch (RevcomCancelled&) {
      } catch (std::exception& e) {
        error = e.what();
      }
      std::lock_guard<std::mutex> lk(m);
      state = DONE;
      cv.notify_all();
    });
  }
  void resume() {
    std::lock_guard<std::mutex> lk(m);
    state = RUNNING;
    cv.notify_all();
  }
  // wait for the next request or the end; true when finished
  bool wait() {
    std::unique_lock<std::mutex> lk(m);
    cv.wait(lk, [&] { return state == REQUEST || state == DONE; });
    if (state == DONE) {
      lk.unlock();
      if (th.joinable()) th.join();
      state = IDLE;
      return true;
    }
    return false;
  }
  void finish_old() {
    if (th.joinable()) {
      {
        std::lock_guard<std::mutex> lk(m);
        cancel = true;
        cv.notify_all();
      }
      th.join();
    }
    state = IDLE;
  }
  ~Revcom() { finish_old(); }
};
template <class T> Revcom& RC() {
  static Revcom r;
  return r;
}

// matvec/precond request wrappers: device <-> caller's X around each request,
// or (device mode) the request is served in place on the device copy of X,
// whose vectors are complete when the request is posted.
template <class T>
std::function<void(int, long, long, long)> revcom_matvec(Revcom& rc, typename HostOf<T>::type* X, bool gep,
                                                         bool pjd, int n, bool dev) {
  return [&rc, X, gep, pjd, n, dev](int which, long x, long y, long by) {
    Global<T>& g = G<T>();
    T* dX = g.W.dX;
    auto st = g.W.st;
    if (dev) {
      CK(cudaStreamSynchronize(st));
      int job = which;
      if (!gep && job == 3) job = 1;
      rc.request(job, x, y, by);
      g.n_matvec++;
      return;
    }
    CK(cudaMemcpyAsync(X + x, dX + x, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int job = which;
    if (!gep && job == 3) job = 1;
    rc.request(job, x, y, by);
    if (which == 1 || which == 3) CK(cudaMemcpyAsync(dX + y, X + y, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    if (gep && (which == 1 || which == 4))
      CK(cudaMemcpyAsync(dX + by, X + by, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    g.n_matvec++;
  };
}
template <class T>
std::function<void(long, long)> revcom_precond(Revcom& rc, typename HostOf<T>::type* X, int n, bool dev) {
  return [&rc, X, n, dev](long rhs, long sol) {
    Global<T>& g = G<T>();
    T* dX = g.W.dX;
    auto st = g.W.st;
    if (dev) {
      CK(cudaStreamSynchronize(st));
      rc.request(2, sol, rhs, 0);
      g.n_precond++;
      return;
    }
    CK(cudaMemcpyAsync(X + rhs, dX + rhs, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    rc.request(2, sol, rhs, 0);
    CK(cudaMemcpyAsync(dX + sol, X + sol, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    g.n_precond++;
  };
}

// Algorithmic bytes of one application of a device factor: L and L^H values
// and column indices, row pointers, the permutation and level lists, the
// block-diagonal D, the input/output vectors (float64) and one read and one
// write of the work vector per phase (gather, two sweeps, D, scatter).
// With a dense tail the swept entries are the bulk rows' and the tail's
// external ones, and both tile sets are read once per application.
// rows solved through dense blocks, and the number of blocks, over all levels
template <class S> static double dense_rows(const DevFactor<S>& F) {
  double r = F.m_tail;
  for (const auto& L : F.lev) r += L.m_tail;
  return r;
}
template <class S> static double dense_blocks(const DevFactor<S>& F) {
  double b = (double)F.blocks.size();
  for (const auto& L : F.lev) b += (double)L.blocks.size();
  return b;
}
// bytes of one entry of the outer (double or double complex) vectors of a factor stored as S
template <class S> struct OuterBytes { static constexpr double v = 8; };
template <> struct OuterBytes<zc> { static constexpr double v = 16; };
template <> struct OuterBytes<cc> { static constexpr double v = 16; };
template <> struct OuterBytes<bc> { static constexpr double v = 16; };
// Algorithmic bytes of one application, as the multilevel solve defines
// them: every stored L entry (value and column index) and row pointer read
// once per sweep, D, the coupling blocks F and F^H once each, the
// permutation and the vectors.  Explicit-inverse tiles are an implementation
// choice and are not counted (precond_bytes below counts what is streamed).
template <class S> static double precond_bytes_alg(const DevFactor<S>& F) {
  const double n = F.n, sz = sizeof(S), sv = sizeof(typename DevFactor<S>::A);
  if (F.coupled) {
    double b = 0;
    const int nl = (int)F.lev.size();
    for (int l = 0; l < nl; ++l) b += (l + 1 < nl ? 2.0 : 1.0) * precond_bytes_alg(F.lev[l]);
    return b + 2.0 * (double)F.nnz_f * (sz + 4) + 2.0 * (n + 1) * 8 + n * 4 * 2 + 10.0 * n * OuterBytes<S>::v;
  }
  return 2.0 * (double)F.nnz_l * (sz + 4) + 2.0 * (n + 1) * 8 + n * (1 + 2 * sz) + n * 4 * 2 +
         2.0 * n * OuterBytes<S>::v + 4.0 * n * sv;
}
template <class S> static double precond_bytes(const DevFactor<S>& F) {
  const double n = F.n, sz = sizeof(S), sv = sizeof(typename DevFactor<S>::A);
  if (F.coupled) {
    // levels below the last are solved twice; F and F^H once each; the outer
    // vectors (8 or 16 bytes) gathered, kept, combined and scattered
    double b = 0;
    const int nl = (int)F.lev.size();
    for (int l = 0; l < nl; ++l) b += (l + 1 < nl ? 2.0 : 1.0) * precond_bytes(F.lev[l]);
    return b + 2.0 * (double)F.nnz_f * (sz + 4) + 2.0 * (n + 1) * 8 + n * 4 * 2 + 10.0 * n * OuterBytes<S>::v;
  }
  return (double)F.sweep_entries * (sz + 4) + 2.0 * (n + 1) * 8 + 3.0 * n * 4 + n * (1 + 4 + 2 * sz) +
         2.0 * n * 8 + 8.0 * n * sv + F.tile_bytes;
}

// ---------------------------------------------------- no-allocation path ----
// Device storage of jdgpu_dildl_apply_noalloc: a fixed array in the
// library's device image, present on every GPU that loads the library until
// the process exits.  All calls share it; each call overwrites what it reads.
constexpr size_t kNoallocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Host code cannot use g_noalloc_scratch as a pointer (it names the host-side
// stand-in).  The device address is looked up on every call, with the
// caller's device current: the lookup is cheap, and a cached address would
// go stale when the context is torn down and the module loaded again (for
// example after cudaDeviceReset).
static void* noalloc_scratch_ptr() {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    throw std::runtime_error(std::string("cudaGetSymbolAddress of the scratch array failed: ") +
                             cudaGetErrorString(e));
  return p;
}

struct ScratchFull : std::runtime_error {
  ScratchFull() : std::runtime_error("problem needs more device memory than the 32 MiB scratch array") {}
};
// hands out 256-byte aligned slices of the scratch array
struct ScratchBump {
  unsigned char* base;
  size_t* used;
  void* operator()(size_t bytes) const {
    size_t off = (*used + 255) & ~size_t(255);
    if (off > kNoallocScratchBytes || bytes > kNoallocScratchBytes - off) throw ScratchFull();
    *used = off + bytes;
    return base + off;
  }
};

static void report(const std::exception& e, int* info) {
  std::fprintf(stderr, " JADAMILU-GB300 error: %s\n", e.what());
  *info = -54330;
}

}  // namespace jdg

using namespace jdg;
using zh = std::complex<double>;

// ===================================================== the C / Fortran ABI ====
namespace {

template <class T>
void pjd_entry(int* N, typename HostOf<T>::type* A, int* JA, int* IA, typename HostOf<T>::type* B, int* JB, int* IB,
               double* EIGS, double* RES, typename HostOf<T>::type* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
               int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
               int* ICNTL, int* IPRINT, int* INFO, double* GAP, bool gep) {
  int keep = ICNTL[0];
  ICNTL[0] = 1;
  try {
    pjd_drive<T>(*N, A, JA, IA, B, JB, IB, EIGS, RES, X, *LX, NEIG, *SIGMA, *ISEARCH, *NINIT, *MADSPACE, ITER, *TOL,
                 SHIFT, DROPTOL, MEM, ICNTL, *IPRINT, INFO, GAP, gep, nullptr);
  } catch (std::exception& e) {
    report(e, INFO);
  }
  ICNTL[0] = keep;
}

template <class T>
void pjdrevcom_entry(int* N, typename HostOf<T>::type* A, int* JA, int* IA, typename HostOf<T>::type* B, int* JB,
                     int* IB, double* EIGS, double* RES, typename HostOf<T>::type* X, int* LX, int* NEIG,
                     double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                     double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3,
                     int* IPRINT, int* INFO, double* GAP, bool gep) {
  Revcom& rc = RC<T>();
  if (*IJOB == 0) {
    rc.device = g_opt.revcom_device != 0;
    auto mv = revcom_matvec<T>(rc, X, gep, true, *N, rc.device);
    rc.start([=] {
      pjd_drive<T>(*N, A, JA, IA, B, JB, IB, EIGS, RES, X, *LX, NEIG, *SIGMA, *ISEARCH, *NINIT, *MADSPACE, ITER,
                   *TOL, SHIFT, DROPTOL, MEM, ICNTL, *IPRINT, INFO, GAP, gep, mv);
    });
  } else {
    rc.resume();
  }
  if (rc.wait()) {
    if (!rc.error.empty()) report(std::runtime_error(rc.error), INFO);
    *IJOB = 0;
    return;
  }
  *IJOB = rc.ijob;
  *NDX1 = rc.ndx1;
  *NDX2 = rc.ndx2;
  if (NDX3) *NDX3 = rc.ndx3;
}

template <class T>
void jdrevcom_entry(int* N, double* EIGS, double* RES, typename HostOf<T>::type* X, int* LX, int* NEIG, double* SIGMA,
                    int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2,
                    int* NDX3, int* IPRINT, int* INFO, double* GAP, bool gep) {
  Revcom& rc = RC<T>();
  if (*IJOB == 0) {
    rc.device = g_opt.revcom_device != 0;
    auto mv = revcom_matvec<T>(rc, X, gep, false, *N, rc.device);
    auto pc = revcom_precond<T>(rc, X, *N, rc.device);
    rc.start([=] {
      jd_drive<T>(*N, EIGS, RES, X, *LX, NEIG, *SIGMA, *ISEARCH, *NINIT, *MADSPACE, ITER, *TOL, *IPRINT, INFO, GAP,
                  gep, mv, pc);
    });
  } else {
    rc.resume();
  }
  if (rc.wait()) {
    if (!rc.error.empty()) report(std::runtime_error(rc.error), INFO);
    *IJOB = 0;
    return;
  }
  *IJOB = rc.ijob;
  *NDX1 = rc.ndx1;
  *NDX2 = rc.ndx2;
  if (NDX3) *NDX3 = rc.ndx3;
}

// Device address of X(1) and the stream of the reverse-communication solve
// that is waiting on a request in device mode (see the header).
template <class T> int revcom_device_ptr(void** xd, void** stream) {
  Revcom& rc = RC<T>();
  {
    std::lock_guard<std::mutex> lk(rc.m);
    if (!rc.device || rc.state != Revcom::REQUEST) return -1;
  }
  Global<T>& g = G<T>();
  if (xd) *xd = (void*)g.W.dX;
  if (stream) *stream = (void*)g.W.st;
  return 0;
}
template <class T> void cleanup_entry() {
  RC<T>().finish_old();
  G<T>().cleanup1();
}

}  // namespace

// The reference-named entry points keep their names, or, compiled with
// JDG_ILP64_INNER for the 64-bit-integer library, take an internal prefix and
// sit behind the wrappers of ilp64.cpp.
#ifdef JDG_ILP64_INNER
#define JDG_REF(name) jdg_i32_##name
#else
#define JDG_REF(name) name
#endif

extern "C" {

JDG_API void JDG_REF(dpjd_)(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                   double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                   double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP) {
  pjd_entry<double>(N, A, JA, IA, nullptr, nullptr, nullptr, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE,
                    ITER, TOL, SHIFT, DROPTOL, MEM, ICNTL, IPRINT, INFO, GAP, false);
}
JDG_API void JDG_REF(dpjd_gep_)(int* N, double* A, int* JA, int* IA, double* B, int* JB, int* IB, double* EIGS, double* RES,
                       double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE,
                       int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT,
                       int* INFO, double* GAP) {
  pjd_entry<double>(N, A, JA, IA, B, JB, IB, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL,
                    SHIFT, DROPTOL, MEM, ICNTL, IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(dpjdrevcom_)(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX,
                         int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL,
                         double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2,
                         int* IPRINT, int* INFO, double* GAP) {
  pjdrevcom_entry<double>(N, A, JA, IA, nullptr, nullptr, nullptr, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT,
                          MADSPACE, ITER, TOL, SHIFT, DROPTOL, MEM, ICNTL, IJOB, NDX1, NDX2, nullptr, IPRINT, INFO,
                          GAP, false);
}
JDG_API void JDG_REF(dpjdrevcom_gep_)(int* N, double* A, int* JA, int* IA, double* B, int* JB, int* IB, double* EIGS,
                             double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT,
                             int* MADSPACE, int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM,
                             int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* NDX3, int* IPRINT, int* INFO,
                             double* GAP) {
  pjdrevcom_entry<double>(N, A, JA, IA, B, JB, IB, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL,
                          SHIFT, DROPTOL, MEM, ICNTL, IJOB, NDX1, NDX2, NDX3, IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(djdrevcom_)(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
                        int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2,
                        int* IPRINT, int* INFO, double* GAP) {
  jdrevcom_entry<double>(N, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, IJOB, NDX1, NDX2,
                         nullptr, IPRINT, INFO, GAP, false);
}
JDG_API void JDG_REF(djdrevcom_gep_)(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, double* GAP) {
  jdrevcom_entry<double>(N, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, IJOB, NDX1, NDX2,
                         NDX3, IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(dpjdcleanup_)(void) { cleanup_entry<double>(); }

// Legacy entry points (PJD, PJDREVCOM, JDREVCOM, PJDCLEANUP): the real drivers
// with ICNTL(5) forced to 0 (float64 preconditioner), ICNTL(1..4) passed
// through and copied back.  The forced copy is static because a
// reverse-communication solve keeps using it between calls.
static int g_legacy_icntl[5];
static void legacy_in(const int* ICNTL) {
  for (int i = 0; i < 4; ++i) g_legacy_icntl[i] = ICNTL[i];
  g_legacy_icntl[4] = 0;
}
static void legacy_out(int* ICNTL) {
  for (int i = 0; i < 4; ++i) ICNTL[i] = g_legacy_icntl[i];
}
JDG_API void JDG_REF(pjd_)(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                  double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                  double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP) {
  legacy_in(ICNTL);
  JDG_REF(dpjd_)(N, A, JA, IA, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, SHIFT, DROPTOL, MEM,
        g_legacy_icntl, IPRINT, INFO, GAP);
  legacy_out(ICNTL);
}
JDG_API void JDG_REF(pjdrevcom_)(int* N, double* A, int* JA, int* IA, double* EIGS, double* RES, double* X, int* LX, int* NEIG,
                        double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                        double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                        int* INFO, double* GAP) {
  legacy_in(ICNTL);
  JDG_REF(dpjdrevcom_)(N, A, JA, IA, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, SHIFT, DROPTOL, MEM,
              g_legacy_icntl, IJOB, NDX1, NDX2, IPRINT, INFO, GAP);
  legacy_out(ICNTL);
}
JDG_API void JDG_REF(jdrevcom_)(int* N, double* EIGS, double* RES, double* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
                       int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                       int* INFO, double* GAP) {
  JDG_REF(djdrevcom_)(N, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, IJOB, NDX1, NDX2, IPRINT, INFO,
             GAP);
}
JDG_API void JDG_REF(pjdcleanup_)(void) { JDG_REF(dpjdcleanup_)(); }

JDG_API void JDG_REF(zpjd_)(int* N, zh* A, int* JA, int* IA, double* EIGS, double* RES, zh* X, int* LX, int* NEIG,
                   double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                   double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO, double* GAP) {
  pjd_entry<zc>(N, A, JA, IA, nullptr, nullptr, nullptr, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE,
                ITER, TOL, SHIFT, DROPTOL, MEM, ICNTL, IPRINT, INFO, GAP, false);
}
JDG_API void JDG_REF(zpjd_gep_)(int* N, zh* A, int* JA, int* IA, zh* B, int* JB, int* IB, double* EIGS, double* RES, zh* X,
                       int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER,
                       double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IPRINT, int* INFO,
                       double* GAP) {
  pjd_entry<zc>(N, A, JA, IA, B, JB, IB, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, SHIFT,
                DROPTOL, MEM, ICNTL, IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(zpjdrevcom_)(int* N, zh* A, int* JA, int* IA, double* EIGS, double* RES, zh* X, int* LX, int* NEIG,
                         double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, double* SHIFT,
                         double* DROPTOL, double* MEM, int* ICNTL, int* IJOB, int* NDX1, int* NDX2, int* IPRINT,
                         int* INFO, double* GAP) {
  pjdrevcom_entry<zc>(N, A, JA, IA, nullptr, nullptr, nullptr, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT,
                      MADSPACE, ITER, TOL, SHIFT, DROPTOL, MEM, ICNTL, IJOB, NDX1, NDX2, nullptr, IPRINT, INFO, GAP,
                      false);
}
JDG_API void JDG_REF(zpjdrevcom_gep_)(int* N, zh* A, int* JA, int* IA, zh* B, int* JB, int* IB, double* EIGS, double* RES,
                             zh* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH, int* NINIT, int* MADSPACE,
                             int* ITER, double* TOL, double* SHIFT, double* DROPTOL, double* MEM, int* ICNTL, int* IJOB,
                             int* NDX1, int* NDX2, int* NDX3, int* IPRINT, int* INFO, double* GAP) {
  pjdrevcom_entry<zc>(N, A, JA, IA, B, JB, IB, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL,
                      SHIFT, DROPTOL, MEM, ICNTL, IJOB, NDX1, NDX2, NDX3, IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(zjdrevcom_)(int* N, double* EIGS, double* RES, zh* X, int* LX, int* NEIG, double* SIGMA, int* ISEARCH,
                        int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1, int* NDX2,
                        int* IPRINT, int* INFO, double* GAP) {
  jdrevcom_entry<zc>(N, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, IJOB, NDX1, NDX2, nullptr,
                     IPRINT, INFO, GAP, false);
}
JDG_API void JDG_REF(zjdrevcom_gep_)(int* N, double* EIGS, double* RES, zh* X, int* LX, int* NEIG, double* SIGMA,
                            int* ISEARCH, int* NINIT, int* MADSPACE, int* ITER, double* TOL, int* IJOB, int* NDX1,
                            int* NDX2, int* NDX3, int* IPRINT, int* INFO, double* GAP) {
  jdrevcom_entry<zc>(N, EIGS, RES, X, LX, NEIG, SIGMA, ISEARCH, NINIT, MADSPACE, ITER, TOL, IJOB, NDX1, NDX2, NDX3,
                     IPRINT, INFO, GAP, true);
}
JDG_API void JDG_REF(zpjdcleanup_)(void) { cleanup_entry<zc>(); }

// ------------------------------------------------ kernel-level entries ----
JDG_API int jdgpu_device_count(void) {
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) return 0;
  return c;
}

// y = A x with A given like DPJD's (upper, 1-based); x, y host arrays.
JDG_API int jdgpu_dspmv(int n, const int* ia, const int* ja, const double* a, const double* x, double* y) {
  try {
    cudaStream_t st = nullptr;
    SellMatrix<double> M;
    build_sell<double>(n, ia, ja, a, M, st);
    double *dx, *dy;
    CK(cudaMalloc(&dx, sizeof(double) * n));
    CK(cudaMalloc(&dy, sizeof(double) * n));
    CK(cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice));
    k::spmv<double>(M, dx, dy, st);
    CK(cudaGetLastError());
    CK(cudaMemcpy(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost));
    cudaFree(dx);
    cudaFree(dy);
    free_sell(M);
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dspmv: %s\n", e.what());
    return -1;
  }
}
JDG_API int jdgpu_zspmv(int n, const int* ia, const int* ja, const zh* a, const zh* x, zh* y) {
  try {
    cudaStream_t st = nullptr;
    SellMatrix<zc> M;
    build_sell<zc>(n, ia, ja, a, M, st);
    zc *dx, *dy;
    CK(cudaMalloc(&dx, sizeof(zc) * n));
    CK(cudaMalloc(&dy, sizeof(zc) * n));
    CK(cudaMemcpy(dx, x, sizeof(zc) * n, cudaMemcpyHostToDevice));
    k::spmv<zc>(M, dx, dy, st);
    CK(cudaGetLastError());
    CK(cudaMemcpy(y, dy, sizeof(zc) * n, cudaMemcpyDeviceToHost));
    cudaFree(dx);
    cudaFree(dy);
    free_sell(M);
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_zspmv: %s\n", e.what());
    return -1;
  }
}

// Factor A - shift*I on the host (project ILDLC) and apply it on the GPU to
// nrhs right-hand sides: x = P (L D L^T)^{-1} P^T b, |D| when spd != 0;
// precision 0: float64 factor, 1: float32, 2: bfloat16 storage.
JDG_API int jdgpu_dildl_apply(int n, const int* ia, const int* ja, const double* a, double shift, double droptol,
                              double condest, int spd, int precision, int nrhs, const double* b, double* x,
                              long* info) {
  try {
    IldlcParams p;
    p.droptol = droptol;
    p.condest = condest;
    p.mem = 0;
    factor_options(p, n);
    IldlcFactor<double> F;
    int ierr = ildlc_factor<double>(n, ia, ja, a, shift, nullptr, nullptr, nullptr, p, F);
    if (ierr) return ierr;
    cudaStream_t st = nullptr;
    double *db, *dx;
    CK(cudaMalloc(&db, sizeof(double) * n));
    CK(cudaMalloc(&dx, sizeof(double) * n));
    DevFactor<double> Fd;
    DevFactor<float> Fs;
    DevFactor<__nv_bfloat16> Fb;
    // with the "apply_graph" option the application goes through the captured
    // graph on a stream of its own, as inside the eigensolver
    const bool graph = g_opt.apply_graph != 0;
    if (graph) CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (precision == 1) upload_factor(F, Fs, st);
    else if (precision == 2) upload_factor(F, Fb, st);
    else upload_factor(F, Fd, st);
    for (int r = 0; r < nrhs; ++r) {
      CK(cudaMemcpy(db, b + (size_t)r * n, sizeof(double) * n, cudaMemcpyHostToDevice));
      if (graph) {
        if (precision == 1) k::ildl_apply_graph<double, float>(Fs, spd != 0, db, dx, st);
        else if (precision == 2) k::ildl_apply_graph<double, __nv_bfloat16>(Fb, spd != 0, db, dx, st);
        else k::ildl_apply_graph<double, double>(Fd, spd != 0, db, dx, st);
        CK(cudaStreamSynchronize(st));
      } else {
        if (precision == 1) k::ildl_apply<double, float>(Fs, spd != 0, db, dx, st);
        else if (precision == 2) k::ildl_apply<double, __nv_bfloat16>(Fb, spd != 0, db, dx, st);
        else k::ildl_apply<double, double>(Fd, spd != 0, db, dx, st);
      }
      CK(cudaGetLastError());
      CK(cudaMemcpy(x + (size_t)r * n, dx, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    if (graph) CK(cudaStreamDestroy(st));
    if (info) {
      info[0] = (long)F.li.size();
      info[1] = F.nneg;
      info[2] = (long)F.level_start.size() - 1;
      std::vector<int> fp, fr, bp, br;
      ildlc_levels(F, fp, fr, bp, br);
      info[3] = (long)fp.size() - 1;
      info[4] = (long)bp.size() - 1;
    }
    free_factor(Fd);
    free_factor(Fs);
    free_factor(Fb);
    cudaFree(db);
    cudaFree(dx);
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dildl_apply: %s\n", e.what());
    return -99;
  }
}

// Times `reps` applications of the factor of A - shift*I on the GPU (CUDA
// events on the launching stream, graph launches, input resident on the
// device).  out: [0] mean ms per application, [1] nnz(L), [2] forward depth,
// [3] backward depth, [4] launches per application, [5] factor seconds.
JDG_API int jdgpu_dildl_bench(int n, const int* ia, const int* ja, const double* a, double shift, double droptol,
                              double condest, int spd, int precision, int reps, double* out) {
  try {
    IldlcParams p;
    p.droptol = droptol;
    p.condest = condest;
    p.mem = 0;
    factor_options(p, n);
    IldlcFactor<double> F;
    double t0 = wall();
    int ierr = ildlc_factor<double>(n, ia, ja, a, shift, nullptr, nullptr, nullptr, p, F);
    double tf = wall() - t0;
    if (ierr) return ierr;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double *db, *dx;
    CK(cudaMalloc(&db, sizeof(double) * n));
    CK(cudaMalloc(&dx, sizeof(double) * n));
    std::vector<double> hb(n, 1.0);
    CK(cudaMemcpy(db, hb.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    DevFactor<double> Fd;
    DevFactor<float> Fs;
    DevFactor<__nv_bfloat16> Fb;
    auto run = [&]() {
      if (precision == 1) k::ildl_apply_graph<double, float>(Fs, spd != 0, db, dx, st);
      else if (precision == 2) k::ildl_apply_graph<double, __nv_bfloat16>(Fb, spd != 0, db, dx, st);
      else k::ildl_apply_graph<double, double>(Fd, spd != 0, db, dx, st);
    };
    const double tu0 = wall();
    if (precision == 1) upload_factor(F, Fs, st);
    else if (precision == 2) upload_factor(F, Fb, st);
    else upload_factor(F, Fd, st);
    const double tu = wall() - tu0;
    for (int r = 0; r < 3; ++r) run();
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) run();
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    const int g = spd != 0 ? 1 : 0;
    const long long launches = precision == 1 ? Fs.graph_kernels[g] : precision == 2 ? Fb.graph_kernels[g]
                                                                                     : Fd.graph_kernels[g];
    out[0] = ms / reps;
    out[1] = (double)F.li.size();
    {
      std::vector<int> fp, fr, bp, br;
      ildlc_levels(F, fp, fr, bp, br);
      out[2] = (double)fp.size() - 1;
      out[3] = (double)bp.size() - 1;
    }
    out[4] = (double)launches;
    out[6] = precision == 1 ? dense_rows(Fs) : precision == 2 ? dense_rows(Fb) : dense_rows(Fd);
    out[5] = tf;
    out[7] = tu;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    free_factor(Fd);
    free_factor(Fs);
    free_factor(Fb);
    cudaFree(db);
    cudaFree(dx);
    cudaStreamDestroy(st);
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dildl_bench: %s\n", e.what());
    return -99;
  }
}

// Device-resident operation for benchmarking and repeated solves: the matrix
// is expanded and uploaded once; dpjd_ calls then reuse it (and leave the
// eigenvectors on the device) until jdgpu_drelease_matrix.
JDG_API int jdgpu_dprepare_matrix(int n, const int* ia, const int* ja, const double* a) {
  try {
    Global<double>& g = G<double>();
    g.W.ensure(n, n);
    build_sell<double>(n, ia, ja, a, g.A, g.W.st);
    g.resident = true;
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dprepare_matrix: %s\n", e.what());
    return -99;
  }
}
JDG_API void jdgpu_drelease_matrix(void) {
  Global<double>& g = G<double>();
  g.resident = false;
  free_sell(g.A);
}
// Run the solver on a caller-provided CUDA stream (cudaStream_t), e.g. one
// owned by a timing harness; NULL restores the library's own stream.
JDG_API void jdgpu_set_stream(void* stream) {
  G<double>().W.set_stream((cudaStream_t)stream);
  G<zc>().W.set_stream((cudaStream_t)stream);
}
// bytes of the device matrix (SELL storage incl. padding) and its nnz
JDG_API void jdgpu_dmatrix_info(long* out) {
  Global<double>& g = G<double>();
  out[0] = g.A.nnz;
  out[1] = g.A.stored;
  out[2] = g.A.n;
}

JDG_API long long jdgpu_launch_count(void) { return k::launch_count(); }

// Times `reps` applications of the last solve's device factor (T: the outer
// arithmetic, double or complex double) through its captured graph.  out: ms
// per application, bytes streamed, nnz(L), rows in dense blocks, kernels per
// application, algorithmic bytes.
extern "C++" {
template <class T> static int precond_bench(int reps, double* out) {
  Global<T>& g = G<T>();
  if (g.factdgl >= 0) return -1;
  const long n = g.F.n;
  cudaStream_t st = g.W.st;
  T *b, *x;
  CK(cudaMalloc(&b, sizeof(T) * n));
  CK(cudaMalloc(&x, sizeof(T) * n));
  k::fill<T>(n, T(1.0), b, st);
  auto run = [&]() {
    if (g.precision == 1) k::ildl_apply_graph<T, typename Global<T>::L>(g.Fs, false, b, x, st);
    else if (g.precision == 2) k::ildl_apply_graph<T, typename Global<T>::B>(g.Fb, false, b, x, st);
    else k::ildl_apply_graph<T, T>(g.Fd, false, b, x, st);
  };
  for (int r = 0; r < 2; ++r) run();
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, st));
  for (int r = 0; r < reps; ++r) run();
  CK(cudaEventRecord(e1, st));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  out[0] = ms / reps;
  auto fill_out = [&](const auto& D) {
    out[1] = precond_bytes(D);
    out[2] = (double)D.nnz_l;
    out[3] = dense_rows(D);
    out[4] = (double)D.graph_kernels[0];
    out[5] = precond_bytes_alg(D);
  };
  if (g.precision == 1) fill_out(g.Fs);
  else if (g.precision == 2) fill_out(g.Fb);
  else fill_out(g.Fd);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(b);
  cudaFree(x);
  return 0;
}
}  // extern "C++"
JDG_API int jdgpu_dprecond_bench(int reps, double* out) {
  try {
    return precond_bench<double>(reps, out);
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dprecond_bench: %s\n", e.what());
    return -99;
  }
}
JDG_API int jdgpu_zprecond_bench(int reps, double* out) {
  try {
    return precond_bench<zc>(reps, out);
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_zprecond_bench: %s\n", e.what());
    return -99;
  }
}

// Times `reps` SpMVs with the last solve's (or the resident) matrix.  out: ms
// per SpMV, algorithmic bytes (full-matrix values and column indices, slice
// pointers, x and y), nnz, stored entries.
extern "C++" {
template <class T> static int spmv_bench(int reps, double* out) {
  Global<T>& g = G<T>();
  const long n = g.A.n;
  if (n <= 0) return -1;
  cudaStream_t st = g.W.st;
  T *x, *y;
  CK(cudaMalloc(&x, sizeof(T) * n));
  CK(cudaMalloc(&y, sizeof(T) * n));
  k::fill<T>(n, T(1.0), x, st);
  for (int r = 0; r < 2; ++r) k::spmv<T>(g.A, x, y, st);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, st));
  for (int r = 0; r < reps; ++r) k::spmv<T>(g.A, x, y, st);
  CK(cudaEventRecord(e1, st));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  out[0] = ms / reps;
  out[1] = (double)g.A.nnz * (4.0 + sizeof(T)) + 8.0 * (g.A.nslices + 1) + 2.0 * sizeof(T) * n;
  out[2] = (double)g.A.nnz;
  out[3] = (double)g.A.stored;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  return 0;
}
}  // extern "C++"
JDG_API int jdgpu_dspmv_bench(int reps, double* out) {
  try {
    return spmv_bench<double>(reps, out);
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dspmv_bench: %s\n", e.what());
    return -99;
  }
}
JDG_API int jdgpu_zspmv_bench(int reps, double* out) {
  try {
    return spmv_bench<zc>(reps, out);
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_zspmv_bench: %s\n", e.what());
    return -99;
  }
}

// Copies the host factor of the last real solve out (for a CPU comparison).
// With all pointers NULL returns the sizes in n_out/nnz_out only.
JDG_API int jdgpu_dfactor_export(int* n_out, long long* nnz_out, double* shift_out, int* perm, long long* lp, int* li,
                                 double* lx, signed char* blk, double* dinv, double* doff, double* ainv,
                                 double* aoff) {
  Global<double>& g = G<double>();
  const IldlcFactor<double>& F = g.F;
  *n_out = F.n;
  *nnz_out = (long long)F.li.size();
  *shift_out = g.shift0;
  if (!perm) return 0;
  std::copy(F.perm.begin(), F.perm.end(), perm);
  for (int i = 0; i <= F.n; ++i) lp[i] = F.lp[i];
  std::copy(F.li.begin(), F.li.end(), li);
  std::copy(F.lx.begin(), F.lx.end(), lx);
  std::copy(F.blk.begin(), F.blk.end(), blk);
  std::copy(F.dinv.begin(), F.dinv.end(), dinv);
  std::copy(F.doff.begin(), F.doff.end(), doff);
  std::copy(F.ainv.begin(), F.ainv.end(), ainv);
  std::copy(F.aoff.begin(), F.aoff.end(), aoff);
  return 0;
}

// The level structure and coupling blocks of that factor (see the header).
JDG_API int jdgpu_dfactor_export_levels(int* coupling_out, int* nlev_out, long long* nnzf_out, int* level_start,
                                        long long* fp, int* fi, double* fx) {
  const IldlcFactor<double>& F = G<double>().F;
  *coupling_out = F.coupling;
  *nlev_out = (int)F.level_start.size() - 1;
  *nnzf_out = (long long)F.fi.size();
  if (!level_start) return 0;
  std::copy(F.level_start.begin(), F.level_start.end(), level_start);
  if (F.coupling == 1) {
    for (int i = 0; i <= F.n; ++i) fp[i] = F.fp[i];
    std::copy(F.fi.begin(), F.fi.end(), fi);
    std::copy(F.fx.begin(), F.fx.end(), fx);
  }
  return 0;
}

// The preconditioner application of jdgpu_dildl_apply without any GPU
// memory allocation (see the header).  Returns 0, a factorisation error code,
// -98 when the problem does not fit in the scratch array, -99 on a CUDA error.
JDG_API int jdgpu_dildl_apply_noalloc(int n, const int* ia, const int* ja, const double* a, double shift,
                                      double droptol, double condest, int spd, int precision, int nrhs,
                                      const double* b, double* x, long* info) {
  if (n <= 0 || nrhs < 0 || precision < 0 || precision > 2) return -1;
  try {
    unsigned char* base = (unsigned char*)noalloc_scratch_ptr();
    IldlcParams p;
    p.droptol = droptol;
    p.condest = condest;
    p.mem = 0;
    factor_options(p, n);
    IldlcFactor<double> F;
    int ierr = ildlc_factor<double>(n, ia, ja, a, shift, nullptr, nullptr, nullptr, p, F);
    if (ierr) return ierr;
    cudaStream_t st = nullptr;
    size_t used = 0;
    ScratchBump bump{base, &used};
    double* db = (double*)bump(sizeof(double) * n);
    double* dx = (double*)bump(sizeof(double) * n);
    DevFactor<double> Fd;
    DevFactor<float> Fs;
    DevFactor<__nv_bfloat16> Fb;
    // applied without the captured graph: no graph input/output vectors
    if (precision == 1) upload_factor(F, Fs, st, bump, false);
    else if (precision == 2) upload_factor(F, Fb, st, bump, false);
    else upload_factor(F, Fd, st, bump, false);
    for (int r = 0; r < nrhs; ++r) {
      CK(cudaMemcpy(db, b + (size_t)r * n, sizeof(double) * n, cudaMemcpyHostToDevice));
      if (precision == 1) k::ildl_apply<double, float>(Fs, spd != 0, db, dx, st);
      else if (precision == 2) k::ildl_apply<double, __nv_bfloat16>(Fb, spd != 0, db, dx, st);
      else k::ildl_apply<double, double>(Fd, spd != 0, db, dx, st);
      CK(cudaGetLastError());
      CK(cudaMemcpy(x + (size_t)r * n, dx, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    if (info) {
      info[0] = (long)F.li.size();
      info[1] = F.nneg;
      info[2] = (long)F.level_start.size() - 1;
      std::vector<int> fp, fr, bp, br;
      ildlc_levels(F, fp, fr, bp, br);
      info[3] = (long)fp.size() - 1;
      info[4] = (long)bp.size() - 1;
    }
    // the DevFactor objects point into the scratch array: nothing to free
    return 0;
  } catch (ScratchFull& e) {
    std::fprintf(stderr, "jdgpu_dildl_apply_noalloc: %s\n", e.what());
    return -98;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_dildl_apply_noalloc: %s\n", e.what());
    return -99;
  }
}

JDG_API int jdgpu_revcom_device_ptr(int complex_, void** xd, void** stream) {
  return complex_ ? revcom_device_ptr<zc>(xd, stream) : revcom_device_ptr<double>(xd, stream);
}

JDG_API void jdgpu_set_option(const char* name, double value) {
  if (!std::strcmp(name, "depth_weight")) g_opt.depth_weight = value;
  else if (!std::strcmp(name, "dense_tail")) g_opt.dense_tail = (int)value;
  else if (!std::strcmp(name, "dense_max")) g_opt.dense_max = (int)value;
  else if (!std::strcmp(name, "dense_min_saving")) g_opt.dense_min_saving = value;
  else if (!std::strcmp(name, "plan_launch_us")) g_opt.plan_launch_us = value;
  else if (!std::strcmp(name, "plan_tile_gbs")) g_opt.plan_tile_gbs = value;
  else if (!std::strcmp(name, "drop_schur")) g_opt.drop_schur = value;
  else if (!std::strcmp(name, "pdl")) k::set_pdl(value != 0);
  else if (!std::strcmp(name, "apply_graph")) g_opt.apply_graph = (int)value;
  else if (!std::strcmp(name, "fuse_inner")) g_opt.fuse_inner = (int)value;
  else if (!std::strcmp(name, "revcom_device")) g_opt.revcom_device = (int)value;
  else if (!std::strcmp(name, "matching")) g_opt.matching = (int)value;
  else if (!std::strcmp(name, "verbose")) g_opt.verbose = (int)value;
  else if (!std::strcmp(name, "coupling")) g_opt.coupling = (int)value;
  else if (!std::strcmp(name, "drop_rule")) g_opt.drop_rule = (int)value;
  else if (!std::strcmp(name, "last_droptol")) g_opt.last_droptol = value;
  else if (!std::strcmp(name, "last_fill")) g_opt.last_fill = value;
  else if (!std::strcmp(name, "coupled_min_n")) g_opt.coupled_min_n = (int)value;
  else if (!std::strcmp(name, "large_form_isearch")) g_opt.large_form_isearch = (int)value;
  else if (!std::strcmp(name, "lookahead")) g_opt.lookahead = (int)value;
  else if (!std::strcmp(name, "factor_verbose")) g_opt.factor_verbose = (int)value;
  else if (!std::strcmp(name, "tri_cluster")) g_opt.tri_cluster = (int)value;
  else if (!std::strcmp(name, "dense_min_rows")) g_opt.dense_min_rows = (int)value;
}

// statistics of the last real-arithmetic solve: factor seconds, upload seconds,
// preconditioner applications, matvecs, levels, forward/backward depth, nnz(L)
JDG_API void jdgpu_dstats(double* out) {
  Global<double>& g = G<double>();
  out[0] = g.t_factor;
  out[1] = g.t_upload;
  out[2] = (double)g.n_precond;
  out[3] = (double)g.n_matvec;
  out[4] = g.last_levels;
  out[5] = g.last_fdepth;
  out[6] = g.last_bdepth;
  out[7] = (double)g.F.li.size();
  out[8] = g.F.fill();
  out[9] = g.nfactor;
  out[10] = g.precision == 1 ? dense_rows(g.Fs) : g.precision == 2 ? dense_rows(g.Fb) : dense_rows(g.Fd);
  out[11] = g.precision == 1 ? dense_blocks(g.Fs) : g.precision == 2 ? dense_blocks(g.Fb) : dense_blocks(g.Fd);
}
// the same for the complex solver state
JDG_API void jdgpu_zstats(double* out) {
  Global<zc>& g = G<zc>();
  out[0] = g.t_factor;
  out[1] = g.t_upload;
  out[2] = (double)g.n_precond;
  out[3] = (double)g.n_matvec;
  out[4] = g.last_levels;
  out[5] = g.last_fdepth;
  out[6] = g.last_bdepth;
  out[7] = (double)g.F.li.size();
  out[8] = g.F.fill();
  out[9] = g.nfactor;
  out[10] = g.precision == 1 ? dense_rows(g.Fs) : g.precision == 2 ? dense_rows(g.Fb) : dense_rows(g.Fd);
  out[11] = g.precision == 1 ? dense_blocks(g.Fs) : g.precision == 2 ? dense_blocks(g.Fb) : dense_blocks(g.Fd);
}
JDG_API void jdgpu_reset_stats(void) {
  Global<double>& g = G<double>();
  g.t_factor = g.t_upload = 0;
  g.n_precond = g.n_matvec = 0;
  g.nfactor = 0;
  Global<zc>& z = G<zc>();
  z.t_factor = z.t_upload = 0;
  z.n_precond = z.n_matvec = 0;
  z.nfactor = 0;
}


// Eigenvector-loss gradient (see the header).  The adjoint mu solves
//   P^T (A - lambda B) P mu = P^T g,  P = I - x x^T B,  x^T B mu = 0,
// by preconditioned MINRES (Paige and Saunders' recurrences) with the
// operator and the preconditioner P |L D L^T|^{-1} P^T applied on the GPU:
// the SELL SpMV, B diagonal, and the ILDLC factor of A - lambda B in its
// positive definite |D| form.  grad[q] = -(mu_i x_j + mu_j x_i) for a stored
// off-diagonal entry (i, j), -mu_i x_i on the diagonal.
JDG_API int jdgpu_deigvec_grad(int n, const int* ia, const int* ja, const double* a, const double* bdiag,
                               double lambda, const double* xin, const double* g, double droptol, double tol,
                               int maxit, double* grad, double* out) {
  if (n <= 1 || !ia || !ja || !a || !xin || !g || !grad || maxit < 1) return -1;
  try {
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    SellMatrix<double> Am;
    build_sell<double>(n, ia, ja, a, Am, st);
    IldlcParams p;
    p.droptol = droptol;
    p.condest = 5;
    p.mem = 0;
    factor_options(p, n);
    IldlcFactor<double> F;
    int ierr;
    if (bdiag) {  // A - lambda B with B diagonal: B as its own diagonal CSR
      std::vector<int> ib(n + 1), jb(n);
      for (int i = 0; i <= n; ++i) ib[i] = i + 1;
      for (int i = 0; i < n; ++i) jb[i] = i + 1;
      ierr = ildlc_factor<double>(n, ia, ja, a, lambda, ib.data(), jb.data(), bdiag, p, F);
    } else {
      ierr = ildlc_factor<double>(n, ia, ja, a, lambda, nullptr, nullptr, nullptr, p, F);
    }
    if (ierr) {
      free_sell(Am);
      cudaStreamDestroy(st);
      return ierr;
    }
    DevFactor<double> D;
    upload_factor(F, D, st);
    const size_t vb = sizeof(double) * n;
    enum { X, BX, G, R1, R2, Y, V, W, W1, W2, MU, T1, T2, BD, NV };
    std::vector<double*> vec(NV, nullptr);
    for (int k = 0; k < NV; ++k) CK(cudaMalloc(&vec[k], vb));
    double *dsm, *dpart;
    CK(cudaMalloc(&dsm, sizeof(double) * 4));
    CK(cudaMalloc(&dpart, sizeof(double) * k::mdot_partial_size(n, 1)));
    CK(cudaMemset(dpart, 0, sizeof(double) * k::mdot_partial_size(n, 1)));
    CK(cudaMemcpyAsync(vec[X], xin, vb, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(vec[G], g, vb, cudaMemcpyHostToDevice, st));
    if (bdiag) CK(cudaMemcpyAsync(vec[BD], bdiag, vb, cudaMemcpyHostToDevice, st));
    auto dot = [&](const double* u, const double* w) {
      double h = 0;
      k::mdot<double>(n, 1, u, n, w, dsm, dpart, st);
      CK(cudaMemcpyAsync(&h, dsm, sizeof(double), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      return h;
    };
    auto bmul = [&](const double* u, double* w) {  // w = B u
      if (bdiag) k::diagsolve<double>(n, vec[BD], u, w, st);
      else CK(cudaMemcpyAsync(w, u, vb, cudaMemcpyDeviceToDevice, st));
    };
    // normalise x to x^T B x = 1 (the scale the formula assumes)
    bmul(vec[X], vec[BX]);
    const double xbx = dot(vec[X], vec[BX]);
    if (!(xbx > 0)) throw std::runtime_error("x^T B x is not positive");
    k::scal<double>(n, 1 / std::sqrt(xbx), vec[X], st);
    k::scal<double>(n, 1 / std::sqrt(xbx), vec[BX], st);
    auto proj_t = [&](double* u) {  // u := P^T u = u - B x (x^T u)
      const double c = dot(vec[X], u);
      k::axpy<double>(n, -c, vec[BX], u, st);
    };
    auto proj = [&](double* u) {  // u := P u = u - x (x^T B u)
      const double c = dot(vec[BX], u);
      k::axpy<double>(n, -c, vec[X], u, st);
    };
    auto op = [&](const double* u, double* w) {  // w = P^T (A - lambda B) P u
      CK(cudaMemcpyAsync(vec[T1], u, vb, cudaMemcpyDeviceToDevice, st));
      proj(vec[T1]);
      k::spmv<double>(Am, vec[T1], w, st);
      bmul(vec[T1], vec[T2]);
      k::axpy<double>(n, -lambda, vec[T2], w, st);
      proj_t(w);
    };
    auto prec = [&](const double* u, double* w) {  // w = P |F|^{-1} P^T u
      CK(cudaMemcpyAsync(vec[T1], u, vb, cudaMemcpyDeviceToDevice, st));
      proj_t(vec[T1]);
      k::ildl_apply<double, double>(D, true, vec[T1], w, st);
      proj(w);
    };
    // preconditioned MINRES from mu = 0 on b = P^T g
    CK(cudaMemcpyAsync(vec[R1], vec[G], vb, cudaMemcpyDeviceToDevice, st));
    proj_t(vec[R1]);
    CK(cudaMemcpyAsync(vec[R2], vec[R1], vb, cudaMemcpyDeviceToDevice, st));
    prec(vec[R1], vec[Y]);
    double beta1 = dot(vec[R1], vec[Y]);
    if (beta1 < 0) throw std::runtime_error("the preconditioner is not positive definite");
    beta1 = std::sqrt(beta1);
    for (int k2 : {W, W1, W2, MU}) k::fill<double>(n, 0.0, vec[k2], st);
    double oldb = 0, beta = beta1, dbar = 0, epsln = 0, phibar = beta1, cs = -1, sn = 0, rnorm = beta1;
    int it = 0;
    const double eps = std::numeric_limits<double>::epsilon();
    while (beta1 > 0 && it < maxit) {
      ++it;
      CK(cudaMemcpyAsync(vec[V], vec[Y], vb, cudaMemcpyDeviceToDevice, st));
      k::scal<double>(n, 1 / beta, vec[V], st);
      op(vec[V], vec[Y]);
      if (it >= 2) k::axpy<double>(n, -beta / oldb, vec[R1], vec[Y], st);
      const double alfa = dot(vec[V], vec[Y]);
      k::axpy<double>(n, -alfa / beta, vec[R2], vec[Y], st);
      std::swap(vec[R1], vec[R2]);
      CK(cudaMemcpyAsync(vec[R2], vec[Y], vb, cudaMemcpyDeviceToDevice, st));
      prec(vec[R2], vec[Y]);
      oldb = beta;
      const double bb = dot(vec[R2], vec[Y]);
      if (bb < 0) throw std::runtime_error("the preconditioner is not positive definite");
      beta = std::sqrt(bb);
      const double oldeps = epsln, delta = cs * dbar + sn * alfa, gbar = sn * dbar - cs * alfa;
      epsln = sn * beta;
      dbar = -cs * beta;
      const double gamma = std::max(std::sqrt(gbar * gbar + beta * beta), eps);
      cs = gbar / gamma;
      sn = beta / gamma;
      const double phi = cs * phibar;
      phibar = sn * phibar;
      // w = (v - oldeps w1 - delta w2) / gamma, with w1 <- w2 <- w
      std::swap(vec[W1], vec[W2]);
      std::swap(vec[W2], vec[W]);
      CK(cudaMemcpyAsync(vec[W], vec[V], vb, cudaMemcpyDeviceToDevice, st));
      k::axpy<double>(n, -oldeps, vec[W1], vec[W], st);
      k::axpy<double>(n, -delta, vec[W2], vec[W], st);
      k::scal<double>(n, 1 / gamma, vec[W], st);
      k::axpy<double>(n, phi, vec[W], vec[MU], st);
      rnorm = phibar;
      if (rnorm <= tol * beta1 || beta == 0) break;
    }
    proj(vec[MU]);
    std::vector<double> mu(n), x(n);
    CK(cudaMemcpyAsync(mu.data(), vec[MU], vb, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(x.data(), vec[X], vb, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i)
      for (int q = ia[i] - 1; q < ia[i + 1] - 1; ++q) {
        const int j = ja[q] - 1;
        grad[q] = (i == j) ? -mu[i] * x[i] : -(mu[i] * x[j] + mu[j] * x[i]);
      }
    if (out) {
      out[0] = it;
      out[1] = beta1 > 0 ? rnorm / beta1 : 0;
    }
    for (auto* v : vec) cudaFree(v);
    cudaFree(dsm);
    cudaFree(dpart);
    free_factor(D);
    free_sell(Am);
    cudaStreamDestroy(st);
    return 0;
  } catch (std::exception& e) {
    std::fprintf(stderr, "jdgpu_deigvec_grad: %s\n", e.what());
    return -99;
  }
}

// Batched DPJD (see the header): worker threads, each with its own solver
// state and CUDA stream, take problems largest first.
JDG_API int jdgpu_dpjd_batch(int nprob, const int* n, double* const* a, int* const* ja, int* const* ia,
                             double* const* eigs, double* const* res, double* const* x, const int* lx, int* neig,
                             int* iter, int* info, double* gap, double sigma, int isearch, int madspace, double tol,
                             double droptol, double mem, const int* icntl, int nworkers) {
  if (nprob < 0 || nworkers < 1 || !n || !a || !ja || !ia || !eigs || !res || !x || !lx || !neig || !iter || !info ||
      !icntl)
    return -1;
  std::vector<int> order(nprob);
  for (int q = 0; q < nprob; ++q) order[q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return n[u] > n[v]; });
  const int nw = std::max(1, std::min(nworkers, nprob));
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int ft = std::max(1, hw / nw);
  std::atomic<int> next{0};
  auto work = [&]() {
    Global<double> own;
    own.factor_threads = ft;
    thread_global<double>() = &own;
    for (;;) {
      const int p = next.fetch_add(1);
      if (p >= nprob) break;
      const int q = order[p];
      int N = n[q], LX = lx[q], NEIG = neig[q], ISEARCH = isearch, NINIT = 0, MAD = madspace, ITER = iter[q];
      int IPRINT = 0, INFO = 0;
      int ICN[5] = {icntl[0], 0, icntl[2], icntl[3], icntl[4]};
      double SIGMA = sigma, TOL = tol, SHIFT = 0, DT = droptol, MEM = mem, GAP = 0;
      pjd_entry<double>(&N, a[q], ja[q], ia[q], nullptr, nullptr, nullptr, eigs[q], res[q], x[q], &LX, &NEIG, &SIGMA,
                        &ISEARCH, &NINIT, &MAD, &ITER, &TOL, &SHIFT, &DT, &MEM, ICN, &IPRINT, &INFO, &GAP, false);
      neig[q] = NEIG;
      iter[q] = ITER;
      info[q] = INFO;
      if (gap) gap[q] = GAP;
      own.cleanup1();
    }
    own.release();
    thread_global<double>() = nullptr;
  };
  std::vector<std::thread> th;
  try {
    for (int w = 1; w < nw; ++w) th.emplace_back(work);
  } catch (std::exception& e) {  // fewer threads than asked: the started ones and this one share the work
    std::fprintf(stderr, "jdgpu_dpjd_batch: %s\n", e.what());
  }
  work();
  for (auto& t : th) t.join();
  return 0;
}

}  // extern "C"
