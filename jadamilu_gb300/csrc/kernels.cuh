// Launch wrappers for the sm_103a kernels of the Jacobi-Davidson hot path.
// Every wrapper enqueues on the given stream and never synchronises.
#pragma once
#include <vector>

#include "common.cuh"

namespace jdg {

// Full Hermitian matrix in SELL-32 (slices of 32 rows, column-major inside a
// slice, padded with the row's own index and a zero value).
template <class T> struct SellMatrix {
  int n = 0, nslices = 0;
  int64_t nnz = 0;       // nonzeros of the full matrix (both triangles)
  int64_t stored = 0;    // stored entries including padding
  int64_t* sptr = nullptr;
  int* col = nullptr;
  T* val = nullptr;
};

// A block of consecutive rows [s0, s0 + m) after the bulk levels.  Forward:
// its external entries (columns < s0) are applied, then, when nt > 0, the
// explicit inverse of its diagonal block as nt x nt tiles of 64 x 64 (layout
// in tail_inverse.hpp).  Backward (blocks in reverse order): the entries of
// L^H pointing past the block, then the tiles of the inverse's adjoint.  A
// block with nt = 0 is one dependency level (identity diagonal block).
template <class S> struct DenseBlk {
  int s0 = 0, m = 0, nt = 0;
  int64_t* ep = nullptr; int* ei = nullptr; S* ev = nullptr;   // forward external, rows local
  int64_t* bp = nullptr; int* bi = nullptr; S* bv = nullptr;   // backward external (L^H), rows local
  int64_t nfe = 0, nbe = 0;                                    // entry counts
  S* tf = nullptr; S* tb = nullptr;                            // tiles of Linv and Linv^H
  int* itf = nullptr; int* itb = nullptr;                      // work items, 4 ints each
  int nitf = 0, nitb = 0;
  int tcl = 8;                                                 // CTAs per cluster of the tile product
  int* irf = nullptr; int* irb = nullptr;                      // items of each tile row
};

// Level-scheduled factor on the device, in "solve numbering" s: rows of the
// same forward level are contiguous; L^H rows are listed level by level in
// brows.  S is the storage type, A = Arith<S>::type the arithmetic type.
template <class S> struct DevFactor {
  using A = typename Arith<S>::type;
  int n = 0;
  int64_t nnz_l = 0;
  int* orig = nullptr;                       // orig[s]: row of the input vector
  int64_t* lp = nullptr; int* li = nullptr; S* lx = nullptr;   // forward rows
  int64_t* up = nullptr; int* ui = nullptr; S* ux = nullptr;   // rows of L^H (values conjugated)
  int* brows = nullptr;
  std::vector<int> fptr, bptr;               // level boundaries (host)
  int* dfptr = nullptr; int* dbptr = nullptr; // the same on the device
  // sweep segments: {first level, last level + 1, kind}; kind 1 = one
  // single-CTA launch for the whole run of levels, 8/16/32 = one grid launch
  // for one level with that many lanes per row
  std::vector<int> fseg, bseg;
  signed char* blk = nullptr; int* partner = nullptr;
  S *dv = nullptr, *dof = nullptr, *av = nullptr, *aof = nullptr;  // D^{-1} and |D|^{-1}
  A* y = nullptr;                            // work vector
  // captured launch sequence of one application (per spd flag), reading
  // rhs_in and writing sol_out
  // Tail: rows s >= s_tail (the deepest forward levels, m_tail rows) are
  // solved by one CTA with the tail of y in shared memory.  Forward: the
  // entries of tail rows that point below s_tail ("external") are applied by
  // a grid kernel first; the rest ("internal", local column ids) level by
  // level.  Backward: tail rows depend only on tail rows and are solved first;
  // bptr/brows then list the remaining rows level by level.
  int s_tail = 0, m_tail = 0;
  int64_t* tep = nullptr; int* tei = nullptr; S* tev = nullptr;   // forward external
  int64_t* tip = nullptr; int* tii = nullptr; S* tiv = nullptr;   // forward internal
  int* dtfptr = nullptr; std::vector<int> tfptr;                  // forward tail levels (local rows)
  int64_t* tbp = nullptr; int* tbi = nullptr; S* tbv = nullptr;   // backward tail rows of L^H (local)
  int* dtbptr = nullptr; int* tbrows = nullptr; std::vector<int> tbptr;
  // Dense blocks: when non-empty, the rows s >= s_tail are solved block by
  // block (DenseBlk) instead of by the single-CTA tail kernels.
  std::vector<DenseBlk<S>> blocks;
  A* part = nullptr;                         // per-item partial sums (64 each)
  A* xb = nullptr;                           // right-hand side of the dense block being solved
  int64_t sweep_entries = 0;                 // L / L^H entries the two level sweeps read
  double tile_bytes = 0;                     // bytes of both tile sets
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  long long graph_kernels[2] = {0, 0};
  void* rhs_in = nullptr;
  void* sol_out = nullptr;
  // Multilevel form with coupling blocks (IldlcFactor::coupling == 1): one
  // sub-factor per level (rows in elimination order, identity permutation),
  // the blocks F (rows: steps of the level's pivots; columns: later steps;
  // one CSR over all steps) and, per level l, F_l^H (rows: the steps after
  // level l, row pointers from fhp + fh_row0[l]; columns: the level's steps),
  // and three outer-precision work vectors of n entries.  The fields above
  // then hold only n, nnz_l, graph and the graph's input/output vectors.
  int coupled = 0;
  std::vector<DevFactor<S>> lev;
  std::vector<int> lstart;                   // first step of each level, plus n
  int* perm = nullptr;                       // elimination step -> row of the input vector
  int64_t* fpp = nullptr; int* fpi = nullptr; S* fpx = nullptr;   // F
  int64_t* fhp = nullptr; int* fhi = nullptr; S* fhx = nullptr;   // F^H
  int64_t nnz_f = 0;
  std::vector<int> fp_lanes, fh_lanes;       // lanes per row of each level's F and F^H rows
  std::vector<int64_t> fh_row0;              // first row pointer of each level's F^H block in fhp
  void *cy = nullptr, *cyb = nullptr, *ct = nullptr;
};

namespace k {

// kernels launched by this library so far (graph replays count their kernel nodes)
long long launch_count();
// programmatic dependent launch between the preconditioner's kernels (default on)
void set_pdl(bool on);
void add_launches(long long n);

template <class T> void spmv(const SellMatrix<T>& A, const T* x, T* y, cudaStream_t s);
// y = A x + a x (the shifted operator of the correction equation)
template <class T> void spmv_shift(const SellMatrix<T>& A, T a, const T* x, T* y, cudaStream_t s);
template <class T> void axpy(long n, T a, const T* x, T* y, cudaStream_t s);
// y += sign * (Re *num / Re *den) * x with num and den in device memory
template <class T> void axpy_ratio(long n, const T* num, const T* den, double sign, const T* x, T* y, cudaStream_t s);
// y += (Re *num / Re *den) * x; out = y (out may alias x)
template <class T> void axpy_ratio_copy(long n, const T* num, const T* den, const T* x, T* y, T* out, cudaStream_t s);
// x2 = s (x2 + a p); xc += x2 (axpy, scal, axpy with the same roundings)
template <class T> void smooth(long n, T a, const T* p, double sc, T* x2, T* xc, cudaStream_t s);
template <class T> void scal(long n, double a, T* x, cudaStream_t s);
template <class T> void fill(long n, T v, T* x, cudaStream_t s);
// out[c] = V(:,c)^H w for c < k (deterministic two-pass reduction); partial
// needs mdot_partial_size(n,k) entries
long mdot_partial_size(long n, int k);
template <class T> void mdot(long n, int k, const T* V, long ldv, const T* w, T* out, T* partial, cudaStream_t s);
// w = beta*w + alpha*V*y, y (k <= 64 entries) in device memory or by value
template <class T> void gemv_dev(long n, int k, T alpha, const T* V, long ldv, const T* y, T beta, T* w, cudaStream_t s);
template <class T> void gemv_val(long n, int k, T alpha, const T* V, long ldv, const T* y_host, T beta, T* w, cudaStream_t s);
// out(:,c) = V * Q(:,c), c < keep, Q K x K column-major (host values)
template <class T> void rmult(long n, int K, int keep, const T* V, long ldv, const T* Q_host, T* out, cudaStream_t s);
// sol = d .* rhs (diagonal preconditioner, d real)
template <class T> void diagsolve(long n, const double* d, const T* rhs, T* sol, cudaStream_t s);
// preconditioner application  x = P (L D L^H)^{-1} P^T b  (|D| when spd)
template <class T, class S> void ildl_apply(const DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s);
// the same through the captured graph (builds it on first use); F.rhs_in and
// F.sol_out must hold n entries of T
template <class T, class S> void ildl_apply_graph(DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s);
// lanes of a warp that share one row of a given mean length in the row kernels
int lanes_per_row(double entries_per_row);
// split the level lists of F into wide levels and runs of narrow levels
template <class S, class A> bool tri_cluster16_ok();
template <class S> void ildl_plan(DevFactor<S>& F, const std::vector<int64_t>& lp_host, const std::vector<int64_t>& up_host,
                                  const std::vector<int>& brows_host);
// make the bulk backward sweep start at level 0 (its rows may point into the tail)
template <class S> void ildl_plan_bwd0(DevFactor<S>& F, const std::vector<int64_t>& up_host,
                                      const std::vector<int>& brows_host);

}  // namespace k
}  // namespace jdg
