// sm_103a kernels of the Jacobi-Davidson hot path.
//
// All of them are HBM-bandwidth kernels (no tensor-core work exists on this
// path): SpMV over the full Hermitian matrix in SELL-32 layout (coalesced
// column/value loads), the level-scheduled sweeps of the multilevel LDL^H
// preconditioner, and the BLAS-1/2 vector work of the outer and inner JD
// iterations (deterministic two-pass reductions, so results do not depend on
// the launch).
#include <atomic>

#include <mutex>

#include <cooperative_groups.h>

#include "kernels.cuh"

namespace jdg {
namespace k {

static std::atomic<long long> g_launches{0};
long long launch_count() { return g_launches.load(); }
void add_launches(long long n) { g_launches += n; }
#define COUNT_LAUNCH() (g_launches += 1)

constexpr int TPB = 256;

// Programmatic dependent launch inside the preconditioner graph: a kernel
// lets its successor be scheduled as soon as all of its CTAs have started
// (launch_dependents), and waits for its predecessor to complete and flush
// (griddepcontrol.wait) before reading anything.  Both are no-ops for a
// kernel launched without the attribute.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
// The two halves of pdl_begin, for kernels that load their factor data
// (never written while the preconditioner runs) before waiting for the
// predecessor's results: those loads overlap the predecessor's tail.
__device__ __forceinline__ void pdl_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Asks the TMA unit to bring [p, p + bytes) into L2 and returns at once (a
// hint: nothing waits for it or reads it back).  Only the 16-byte aligned
// interior of the range is requested, in pieces of at most 64 KB, so no byte
// outside [p, p + bytes) is touched.
__device__ __forceinline__ void l2_prefetch(const void* p, size_t bytes) {
  size_t a = __cvta_generic_to_global(p);
  size_t e = a + bytes;
  a = (a + 15) & ~(size_t)15;
  e &= ~(size_t)15;
  while (a < e) {
    const unsigned sz = (unsigned)(e - a < 65536 ? e - a : 65536);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(sz) : "memory");
    a += sz;
  }
}
static bool g_pdl = true;
void set_pdl(bool on) { g_pdl = on; }
template <class... Params, class... Args>
static void launch_k(void (*kern)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl ? 1 : 0;
  CK(cudaLaunchKernelEx(&cfg, kern, static_cast<Params>(args)...));
}
static inline int nblk(long n, int tpb = TPB) { return (int)std::max<long>(1, (n + tpb - 1) / tpb); }

// ---------------------------------------------------------------- SpMV ----
// The first kSellPre entries of a row (SELL-32: entry j of a slice's row at
// 32 j + lane) are loaded before waiting for the predecessor that writes x,
// then gathered together and added in entry order, as one at a time.
constexpr int kSellPre = 8;
template <class T> struct SellBatch {
  int c[kSellPre];
  T v[kSellPre];
};
template <class T>
__device__ __forceinline__ void sell_load(SellBatch<T>& b, int64_t q, int64_t e, const int* __restrict__ col,
                                          const T* __restrict__ val) {
#pragma unroll
  for (int u = 0; u < kSellPre; ++u) {
    const int64_t qq = q + 32 * u;
    if (qq < e) {
      b.c[u] = __ldg(col + qq);
      b.v[u] = val[qq];
    } else {
      b.c[u] = -1;
      b.v[u] = T(0);
    }
  }
}
template <class T> __device__ __forceinline__ T sell_use(const SellBatch<T>& b, const T* __restrict__ x, T acc) {
  T w[kSellPre];
#pragma unroll
  for (int u = 0; u < kSellPre; ++u) w[u] = b.c[u] >= 0 ? x[b.c[u]] : T(0);
#pragma unroll
  for (int u = 0; u < kSellPre; ++u)
    if (b.c[u] >= 0) acc = fma_(b.v[u], w[u], acc);
  return acc;
}
template <class T>
__global__ void __launch_bounds__(TPB) spmv_sell_kernel(int n, const int64_t* __restrict__ sptr,
                                                        const int* __restrict__ col, const T* __restrict__ val,
                                                        const T* __restrict__ x, T* __restrict__ y) {
  pdl_launch();
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int sl = r >> 5, lane = r & 31;
  int64_t b = sptr[sl], e = sptr[sl + 1];
  SellBatch<T> first;
  sell_load(first, b + lane, e, col, val);
  pdl_wait();
  T acc = sell_use(first, x, T(0));
  for (int64_t q = b + lane + kSellPre * 32; q < e; q += 32) acc = fma_(val[q], x[__ldg(col + q)], acc);
  y[r] = acc;
}
template <class T> void spmv(const SellMatrix<T>& A, const T* x, T* y, cudaStream_t s) {
  launch_k(spmv_sell_kernel<T>, dim3(nblk(A.n)), dim3(TPB), 0, s, A.n, A.sptr, A.col, A.val, x, y);
  COUNT_LAUNCH();
}
// y = A x + a x: the row sum, then the same fused multiply-add as axpy
template <class T>
__global__ void __launch_bounds__(TPB) spmv_shift_kernel(int n, const int64_t* __restrict__ sptr,
                                                         const int* __restrict__ col, const T* __restrict__ val,
                                                         T a, const T* __restrict__ x, T* __restrict__ y) {
  pdl_launch();
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int sl = r >> 5, lane = r & 31;
  int64_t b = sptr[sl], e = sptr[sl + 1];
  SellBatch<T> first;
  sell_load(first, b + lane, e, col, val);
  pdl_wait();
  T acc = sell_use(first, x, T(0));
  for (int64_t q = b + lane + kSellPre * 32; q < e; q += 32) acc = fma_(val[q], x[__ldg(col + q)], acc);
  y[r] = fma_(a, x[r], acc);
}
template <class T> void spmv_shift(const SellMatrix<T>& A, T a, const T* x, T* y, cudaStream_t s) {
  launch_k(spmv_shift_kernel<T>, dim3(nblk(A.n)), dim3(TPB), 0, s, A.n, A.sptr, A.col, A.val, a, x, y);
  COUNT_LAUNCH();
}

// -------------------------------------------------------------- BLAS-1 ----
template <class T> __global__ void axpy_kernel(long n, T a, const T* __restrict__ x, T* __restrict__ y) {
  pdl_begin();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = fma_(a, x[i], y[i]);
}
// y += sign * (Re num / Re den) * x, the two scalars read from device memory
// (results of earlier reductions on the same stream)
template <class T>
__global__ void axpy_ratio_kernel(long n, const T* num, const T* den, double sign, const T* __restrict__ x,
                                  T* __restrict__ y) {
  pdl_begin();
  const T a = T(sign * (rl(*num) / rl(*den)));
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = fma_(a, x[i], y[i]);
}
// y += (Re num / Re den) * x, then out = y (out may alias x)
template <class T>
__global__ void axpy_ratio_copy_kernel(long n, const T* num, const T* den, const T* x, T* __restrict__ y, T* out) {
  pdl_begin();
  const T a = T(1.0 * (rl(*num) / rl(*den)));
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T t = fma_(a, x[i], y[i]);
    y[i] = t;
    out[i] = t;
  }
}
// x2 = s (x2 + a p); xc = x2 + xc, as axpy, scal and axpy in sequence
template <class T>
__global__ void smooth_kernel(long n, T a, const T* __restrict__ p, double s, T* __restrict__ x2, T* __restrict__ xc) {
  pdl_begin();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T t = s * fma_(a, p[i], x2[i]);
    x2[i] = t;
    xc[i] = fma_(T(1), t, xc[i]);
  }
}
template <class T> __global__ void scal_kernel(long n, double a, T* x) {
  pdl_begin();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] = a * x[i];
}
template <class T> __global__ void fill_kernel(long n, T v, T* x) {
  pdl_begin();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] = v;
}
static inline int grid_1d(long n) { return (int)std::min<long>(nblk(n), 152L * 16); }
template <class T> void axpy(long n, T a, const T* x, T* y, cudaStream_t s) {
  if (n > 0) { launch_k(axpy_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, a, x, y); COUNT_LAUNCH(); }
}
template <class T>
void axpy_ratio(long n, const T* num, const T* den, double sign, const T* x, T* y, cudaStream_t s) {
  if (n > 0) { launch_k(axpy_ratio_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, num, den, sign, x, y); COUNT_LAUNCH(); }
}
template <class T> void axpy_ratio_copy(long n, const T* num, const T* den, const T* x, T* y, T* out, cudaStream_t s) {
  if (n > 0) { launch_k(axpy_ratio_copy_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, num, den, x, y, out); COUNT_LAUNCH(); }
}
template <class T> void smooth(long n, T a, const T* p, double sc, T* x2, T* xc, cudaStream_t s) {
  if (n > 0) { launch_k(smooth_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, a, p, sc, x2, xc); COUNT_LAUNCH(); }
}
template <class T> void scal(long n, double a, T* x, cudaStream_t s) {
  if (n > 0) { launch_k(scal_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, a, x); COUNT_LAUNCH(); }
}
template <class T> void fill(long n, T v, T* x, cudaStream_t s) {
  if (n > 0) { launch_k(fill_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, v, x); COUNT_LAUNCH(); }
}

// ---------------------------------------------------- reductions (V^H w) ----
__device__ __forceinline__ double shfl_down(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ zc shfl_down(zc v, int o) { return zc(shfl_down(v.x, o), shfl_down(v.y, o)); }
__device__ __forceinline__ float shfl_xor_any(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_xor_any(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ cc shfl_xor_any(cc v, int o) { return cc(shfl_xor_any(v.x, o), shfl_xor_any(v.y, o)); }
__device__ __forceinline__ zc shfl_xor_any(zc v, int o) { return zc(shfl_xor_any(v.x, o), shfl_xor_any(v.y, o)); }

// loads that bypass L1 (data another CTA of the same launch wrote)
__device__ __forceinline__ double ldcg_(const double* p) { return __ldcg(p); }
__device__ __forceinline__ zc ldcg_(const zc* p) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return zc(v.x, v.y);
}

constexpr int MD_CH = 8;  // columns per pass
// Long vectors: up to two rows per thread, enough CTAs in flight to stream V
// at full bandwidth.  Vectors under 4096 rows keep one CTA per 2048 rows, the
// summation order validated on the user-guide samples (n = 1000), whose JD
// trajectories change with the rounding of these inner products.
static inline int md_grid(long n) {
  if (n < 4096) return (int)std::max<long>(1, (n + 2047) / 2048);
  return (int)std::min<long>((n + 511) / 512, 152L * 8);
}

// The partials follow a 16-byte arrival counter at the start of the buffer
// (zero when the buffer is allocated; the last CTA of each call resets it).
constexpr int MD_HEAD = 16;
long mdot_partial_size(long n, int k) {
  return (long)md_grid(n) * ((k + MD_CH - 1) / MD_CH) * MD_CH + 2;  // + the counter (2 doubles or 1 complex)
}

// V^H w in one launch: every CTA writes its per-column partial sums, and the
// CTA that arrives last (a counter, no waiting) adds them per column in the
// fixed order of a second pass (strided over TPB threads, then the warp tree),
// so the result does not depend on which CTA is last.
template <class T>
__global__ void __launch_bounds__(TPB) mdot_kernel(long n, int k, const T* __restrict__ V, long ldv,
                                                   const T* __restrict__ w, unsigned char* __restrict__ buf,
                                                   T* __restrict__ out) {
  pdl_begin();
  unsigned* count = reinterpret_cast<unsigned*>(buf);
  T* partial = reinterpret_cast<T*>(buf + MD_HEAD);
  const int g = gridDim.x;
  const int c0 = blockIdx.y * MD_CH;
  const int nc = min(MD_CH, k - c0);
  T acc[MD_CH];
#pragma unroll
  for (int j = 0; j < MD_CH; ++j) acc[j] = T(0);
  for (long i = blockIdx.x * (long)TPB + threadIdx.x; i < n; i += (long)gridDim.x * TPB) {
    T wi = w[i];
#pragma unroll
    for (int j = 0; j < MD_CH; ++j)
      if (j < nc) acc[j] = fma_(cj(V[i + (long)(c0 + j) * ldv]), wi, acc[j]);
  }
  __shared__ T red[TPB / 32][MD_CH];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < MD_CH; ++j) {
    T v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += shfl_down(v, o);
    if (lane == 0) red[wid][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < MD_CH) {
    T v = T(0);
    for (int q = 0; q < TPB / 32; ++q) v += red[q][threadIdx.x];
    partial[(long)(c0 + threadIdx.x) * g + blockIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(count, 1u) == (unsigned)(g * gridDim.y) - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ T fin[TPB / 32];
  for (int c = 0; c < k; ++c) {
    T v = T(0);
    for (int q = threadIdx.x; q < g; q += TPB) v += ldcg_(partial + (long)c * g + q);
    for (int o = 16; o > 0; o >>= 1) v += shfl_down(v, o);
    if (lane == 0) fin[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      T t = T(0);
      for (int q = 0; q < TPB / 32; ++q) t += fin[q];
      out[c] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = 0u;
}
template <class T> void mdot(long n, int k, const T* V, long ldv, const T* w, T* out, T* partial, cudaStream_t s) {
  if (k <= 0) return;
  int g = md_grid(n);
  dim3 grid(g, (k + MD_CH - 1) / MD_CH);
  launch_k(mdot_kernel<T>, dim3(grid), dim3(TPB), 0, s, n, k, V, ldv, w, reinterpret_cast<unsigned char*>(partial),
           out);
  g_launches += 1;
}

// ------------------------------------------------------ V y (tall-skinny) ----
constexpr int GMV_MAX = 64;
template <class T> struct SmallVec { T v[GMV_MAX]; };

template <class T>
__global__ void __launch_bounds__(TPB) jd_basis_gemv_dev_kernel(long n, int k, T alpha, const T* __restrict__ V, long ldv,
                                                       const T* __restrict__ y, T beta, T* __restrict__ w) {
  pdl_begin();
  __shared__ T ys[GMV_MAX];
  if (threadIdx.x < k) ys[threadIdx.x] = y[threadIdx.x];
  __syncthreads();
  for (long i = blockIdx.x * (long)TPB + threadIdx.x; i < n; i += (long)gridDim.x * TPB) {
    T acc = T(0);
    for (int c = 0; c < k; ++c) acc = fma_(V[i + (long)c * ldv], ys[c], acc);
    T o = (beta == T(0)) ? T(0) : beta * w[i];
    w[i] = fma_(alpha, acc, o);
  }
}
template <class T>
__global__ void __launch_bounds__(TPB) jd_basis_gemv_val_kernel(long n, int k, T alpha, const T* __restrict__ V, long ldv,
                                                       SmallVec<T> y, T beta, T* __restrict__ w) {
  pdl_begin();
  for (long i = blockIdx.x * (long)TPB + threadIdx.x; i < n; i += (long)gridDim.x * TPB) {
    T acc = T(0);
    for (int c = 0; c < k; ++c) acc = fma_(V[i + (long)c * ldv], y.v[c], acc);
    T o = (beta == T(0)) ? T(0) : beta * w[i];
    w[i] = fma_(alpha, acc, o);
  }
}
template <class T>
void gemv_dev(long n, int k, T alpha, const T* V, long ldv, const T* y, T beta, T* w, cudaStream_t s) {
  if (k > GMV_MAX) throw std::runtime_error("gemv_dev: too many columns");
  if (k <= 0) {
    if (!(beta == T(1))) {
      if (beta == T(0)) fill(n, T(0), w, s);
      else throw std::runtime_error("gemv_dev: unsupported beta");
    }
    return;
  }
  launch_k(jd_basis_gemv_dev_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, k, alpha, V, ldv, y, beta, w);
  COUNT_LAUNCH();
}
template <class T>
void gemv_val(long n, int k, T alpha, const T* V, long ldv, const T* yh, T beta, T* w, cudaStream_t s) {
  if (k > GMV_MAX) throw std::runtime_error("gemv_val: too many columns");
  if (k <= 0) {
    if (beta == T(0)) fill(n, T(0), w, s);
    return;
  }
  SmallVec<T> y;
  for (int c = 0; c < k; ++c) y.v[c] = yh[c];
  launch_k(jd_basis_gemv_val_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, k, alpha, V, ldv, y, beta, w);
  COUNT_LAUNCH();
}

// Q (K x keep, leading dimension K, K <= 32) travels in the kernel's
// parameters: at most 16 KB for complex<double>, inside the 32 KB parameter
// space, so a restart needs no staging copy and no host synchronisation.
template <class T> struct SmallMat { T q[32 * 32]; };
template <class T>
__global__ void __launch_bounds__(TPB) rmult_kernel(long n, int K, int keep, const T* __restrict__ V, long ldv,
                                                    const __grid_constant__ SmallMat<T> Q, T* __restrict__ out) {
  pdl_begin();
  __shared__ T qs[32 * 32];
  for (int t = threadIdx.x; t < K * keep; t += TPB) qs[t] = Q.q[t];
  __syncthreads();
  for (long i = blockIdx.x * (long)TPB + threadIdx.x; i < n; i += (long)gridDim.x * TPB) {
    T row[32];
    for (int kk = 0; kk < K; ++kk) row[kk] = V[i + (long)kk * ldv];
    for (int c = 0; c < keep; ++c) {
      T acc = T(0);
      for (int kk = 0; kk < K; ++kk) acc = fma_(row[kk], qs[kk + c * K], acc);
      out[i + (long)c * n] = acc;
    }
  }
}
template <class T> void rmult(long n, int K, int keep, const T* V, long ldv, const T* Qh, T* out, cudaStream_t s) {
  if (K > 32 || keep > K) throw std::runtime_error("rmult: search space above 32");
  SmallMat<T> q;
  for (int c = 0; c < keep; ++c)
    for (int kk = 0; kk < K; ++kk) q.q[kk + c * K] = Qh[kk + c * K];
  launch_k(rmult_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, K, keep, V, ldv, q, out);
  COUNT_LAUNCH();
}

template <class T> __global__ void diag_kernel(long n, const double* __restrict__ d, const T* __restrict__ r, T* x) {
  pdl_begin();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    x[i] = d[i] * r[i];
}
template <class T> void diagsolve(long n, const double* d, const T* rhs, T* sol, cudaStream_t s) {
  launch_k(diag_kernel<T>, dim3(grid_1d(n)), dim3(TPB), 0, s, n, d, rhs, sol);
  COUNT_LAUNCH();
}

// ------------------------------------------------ multilevel LDL^H apply ----
// Entries q, q + step, ... (below e) of a row, U at a time: a batch's
// column indices and values are loaded together, then its gathers of y, and
// the products are added in entry order, so the roundings are those of one
// entry at a time while U dependent load chains are in flight.  kUnr for the
// sweeps; the external-entry gathers of large dense blocks (rows of hundreds
// of entries) take kUnrLong.
constexpr int kUnr = 4;
constexpr int kUnrLong = 8;
template <class A, int U> struct EntBatch {
  int c[U];
  A v[U];
};
template <bool NC, class A, int U, class S>
__device__ __forceinline__ void ent_load(EntBatch<A, U>& b, int64_t q, int64_t e, int step, const int* __restrict__ ci,
                                         const S* __restrict__ cv) {
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t qq = q + (int64_t)u * step;
    if (qq < e) {
      b.c[u] = NC ? ld_idx_nc(ci + qq) : ci[qq];
      b.v[u] = NC ? ldan<A>(cv + qq) : lda<A>(cv + qq);
    } else {
      b.c[u] = -1;
      b.v[u] = A(0);
    }
  }
}
template <class A, int U> __device__ __forceinline__ A ent_use(const EntBatch<A, U>& b, const A* y, A acc) {
  A w[U];
#pragma unroll
  for (int u = 0; u < U; ++u) w[u] = b.c[u] >= 0 ? y[b.c[u]] : A(0);
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (b.c[u] >= 0) acc = fma_(b.v[u], w[u], acc);
  return acc;
}
// entries [q, e) of a row beyond its first batch, into L2 ahead of use
template <class S>
__device__ __forceinline__ void prefetch_rest(int64_t q, int64_t e, const int* __restrict__ ci,
                                              const S* __restrict__ cv) {
  if (q < e) {
    l2_prefetch(ci + q, sizeof(int) * (size_t)(e - q));
    l2_prefetch(cv + q, sizeof(S) * (size_t)(e - q));
  }
}
template <bool NC, int U = kUnr, class A, class S>
__device__ __forceinline__ A ent_dot(int64_t q, int64_t e, int step, const int* __restrict__ ci,
                                     const S* __restrict__ cv, const A* y, A acc) {
  for (; q < e; q += (int64_t)U * step) {
    EntBatch<A, U> b;
    ent_load<NC>(b, q, e, step, ci, cv);
    acc = ent_use(b, y, acc);
  }
  return acc;
}

template <class T, class A>
__global__ void ildl_gather_kernel(int n, const int* __restrict__ orig, const T* __restrict__ b, A* __restrict__ y) {
  pdl_launch();
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int o = orig[s];
  pdl_wait();
  y[s] = cvt<A>(b[o]);
}
template <class T, class A>
__global__ void ildl_scatter_kernel(int n, const int* __restrict__ orig, const A* __restrict__ y, T* __restrict__ x) {
  pdl_launch();
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int o = orig[s];
  pdl_wait();
  x[o] = cvt<T>(y[s]);
}
template <class S, class A>
__global__ void ildl_dsolve_kernel(int n, const signed char* __restrict__ blk, const int* __restrict__ partner,
                                   const S* __restrict__ dv, const S* __restrict__ dof, A* __restrict__ y) {
  pdl_launch();
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  signed char b = blk[s];
  if (b == 1) {
    const A d = lda<A>(dv + s);
    pdl_wait();
    y[s] = d * y[s];
  } else if (b == 2) {
    const int t = partner[s];
    const A o = lda<A>(dof + s), d0 = lda<A>(dv + s), d1 = lda<A>(dv + t);
    pdl_wait();
    A a0 = y[s], a1 = y[t];
    y[s] = fma_(d0, a0, o * a1);
    y[t] = fma_(cj(o), a0, d1 * a1);
  }
}
// A run of narrow levels [l0, l1) in one CTA: a warp per row, levels
// separated by __syncthreads (which orders the CTA's global writes).
__device__ __forceinline__ float wsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ cc wsum(cc v) { return cc(wsum(v.x), wsum(v.y)); }
__device__ __forceinline__ zc wsum(zc v) { return zc(wsum(v.x), wsum(v.y)); }

constexpr int RUN_TPB = 1024;
constexpr int RUN_WARPS = RUN_TPB / 32;
// A level with R < 32 rows gives each row 32/R warps; their partial sums are
// added in a fixed order after a barrier, so results do not depend on timing.
template <class S, class A>
__global__ void __launch_bounds__(RUN_TPB) ildl_run_kernel(int l0, int l1, const int* __restrict__ lptr,
                                                          const int* __restrict__ rows, const int64_t* __restrict__ rp,
                                                          const int* __restrict__ ci, const S* __restrict__ cv,
                                                          A* y) {
  pdl_begin();
  __shared__ A part[RUN_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l = l0; l < l1; ++l) {
    const int lo = lptr[l], hi = lptr[l + 1], R = hi - lo;
    if (R >= RUN_WARPS) {
      for (int t = lo + warp; t < hi; t += RUN_WARPS) {
        const int s = rows ? rows[t] : t;
        const int64_t b = rp[s], e = rp[s + 1];
        A acc = ent_dot<false>(b + lane, e, 32, ci, cv, (const A*)y, A(0));
        acc = wsum(acc);
        if (lane == 0) y[s] = y[s] - acc;
      }
      __syncthreads();
    } else {
      int G = RUN_WARPS / R;
      G = 1 << (31 - __clz(G));
      const int slot = warp / G, sub = warp % G;
      A acc = A(0);
      int s = -1;
      if (slot < R) {
        s = rows ? rows[lo + slot] : lo + slot;
        acc = ent_dot<false>(rp[s] + sub * 32 + lane, rp[s + 1], 32 * G, ci, cv, (const A*)y, acc);
      }
      acc = wsum(acc);
      if (lane == 0) part[warp] = acc;
      __syncthreads();
      if (slot < R && sub == 0 && lane == 0) {
        A t = part[warp];
        for (int j = 1; j < G; ++j) t = t + part[warp + j];
        y[s] = y[s] - t;
      }
      __syncthreads();
    }
  }
}
// One wide level: LANES lanes per row (8, 16 or 32, from the level's mean
// row length, so long rows are read by more lanes at once).
constexpr int WIDE_TPB = 256;
static inline int lanes_for(double entries_per_row) {
  return entries_per_row >= 48 ? 32 : entries_per_row >= 20 ? 16 : 8;
}
int lanes_per_row(double entries_per_row) { return lanes_for(entries_per_row); }
template <class S, class A, int LANES>
__global__ void __launch_bounds__(WIDE_TPB) ildl_wide_kernel(int lo, int hi, const int* __restrict__ rows,
                                                            const int64_t* __restrict__ rp, const int* __restrict__ ci,
                                                            const S* __restrict__ cv, A* __restrict__ y) {
  pdl_launch();
  const int g = blockIdx.x * (WIDE_TPB / LANES) + (threadIdx.x / LANES);
  const int lane = threadIdx.x % LANES;
  const int t = lo + g;
  const bool ok = t < hi;
  int s = 0;
  int64_t b = 0, e = 0;
  if (ok) {
    s = rows ? rows[t] : t;
    b = rp[s] + lane;
    e = rp[s + 1];
    if (lane == 0) prefetch_rest(b + kUnr * LANES, e, ci, cv);
  }
  EntBatch<A, kUnr> first;
  ent_load<false>(first, b, e, LANES, ci, cv);
  pdl_wait();
  A acc = ent_use(first, (const A*)y, A(0));
  acc = ent_dot<false>(b + kUnr * LANES, e, LANES, ci, cv, (const A*)y, acc);
  for (int o = LANES / 2; o > 0; o >>= 1) acc = acc + shfl_xor_any(acc, o);
  if (ok && lane == 0) y[s] = y[s] - acc;
}

// Rows [s0, s0 + m) of a block: y[s0 + t] -= sum of row t's entries (local
// row pointers, global columns), LANES lanes per row.
// out[t] = y[s0 + t] - sum of row t's entries (out may be y + s0).  NC: the
// entries and column indices are read without L1 allocation, which keeps L1
// for the gathered y; measured on GB300 it pays for blocks with a million or
// more external entries (Anderson 50^3 application 0.387 -> 0.356 ms with it
// on every block) and costs a little on smaller ones (40^3: 0.198 -> 0.202).
template <class S, class A, int LANES, bool NC>
__global__ void __launch_bounds__(WIDE_TPB) tail_ext_kernel(int m, int s_tail, const int64_t* __restrict__ rp,
                                                           const int* __restrict__ ci, const S* __restrict__ cv,
                                                           const A* y, A* out) {
  pdl_launch();
  constexpr int U = NC ? kUnrLong : kUnr;
  const int t = blockIdx.x * (WIDE_TPB / LANES) + (threadIdx.x / LANES);
  const int lane = threadIdx.x % LANES;
  int64_t b = 0, e = 0;
  if (t < m) {
    b = rp[t] + lane;
    e = rp[t + 1];
    if (lane == 0) prefetch_rest(b + U * LANES, e, ci, cv);
  }
  EntBatch<A, U> first;
  ent_load<NC>(first, b, e, LANES, ci, cv);
  pdl_wait();
  A acc = ent_use(first, y, A(0));
  acc = ent_dot<NC, U>(b + U * LANES, e, LANES, ci, cv, y, acc);
  for (int o = LANES / 2; o > 0; o >>= 1) acc = acc + shfl_xor_any(acc, o);
  if (t < m && lane == 0) out[t] = y[s_tail + t] - acc;
}
template <class S, class A>
static void launch_wide(int lanes, int lo, int hi, const int* rows, const int64_t* rp, const int* ci, const S* cv, A* y,
                        cudaStream_t s) {
  const int nb = (hi - lo) * lanes / WIDE_TPB + 1;
  if (lanes == 32) launch_k(ildl_wide_kernel<S, A, 32>, dim3(nb), dim3(WIDE_TPB), 0, s, lo, hi, rows, rp, ci, cv, y);
  else if (lanes == 16) launch_k(ildl_wide_kernel<S, A, 16>, dim3(nb), dim3(WIDE_TPB), 0, s, lo, hi, rows, rp, ci, cv, y);
  else launch_k(ildl_wide_kernel<S, A, 8>, dim3(nb), dim3(WIDE_TPB), 0, s, lo, hi, rows, rp, ci, cv, y);
}
constexpr int64_t kExtStreamEntries = 1 << 20;  // external entries from which tail_ext streams them
template <class S, class A, bool NC>
static void launch_ext_(int lanes, int m, int s0, const int64_t* rp, const int* ci, const S* cv, const A* y, A* out,
                        cudaStream_t s) {
  const int nb = m * lanes / WIDE_TPB + 1;
  if (lanes == 32) launch_k(tail_ext_kernel<S, A, 32, NC>, dim3(nb), dim3(WIDE_TPB), 0, s, m, s0, rp, ci, cv, y, out);
  else if (lanes == 16) launch_k(tail_ext_kernel<S, A, 16, NC>, dim3(nb), dim3(WIDE_TPB), 0, s, m, s0, rp, ci, cv, y, out);
  else launch_k(tail_ext_kernel<S, A, 8, NC>, dim3(nb), dim3(WIDE_TPB), 0, s, m, s0, rp, ci, cv, y, out);
}
template <class S, class A>
static void launch_ext(int lanes, int m, int s0, const int64_t* rp, const int* ci, const S* cv, A* y, A* out,
                       int64_t entries, cudaStream_t s) {
  if (entries >= kExtStreamEntries) launch_ext_<S, A, true>(lanes, m, s0, rp, ci, cv, y, out, s);
  else launch_ext_<S, A, false>(lanes, m, s0, rp, ci, cv, y, out, s);
}
// The sequential part of a tail sweep in one CTA.  Shared memory holds the
// tail of y (yt), the row pointers relative to the first tail entry, the level
// pointers and (backward sweep) the row order, so a level costs one global
// load of entries, which is issued for the next level before the barrier.
// Rows of small levels are split over several warps as in ildl_run_kernel.
template <class A> __host__ __device__ constexpr size_t tail_smem_bytes(int m, int nlev, bool rows) {
  return ((sizeof(A) * (size_t)m + 15) / 16) * 16 + 4 * (size_t)(m + 1) + 4 * (size_t)(nlev + 1) +
         (rows ? 4 * (size_t)m : 0);
}
template <class S, class A>
__global__ void __launch_bounds__(RUN_TPB) tail_run_kernel(int m, int s_tail, int nlev, const int* __restrict__ lptr,
                                                          const int* __restrict__ rows, const int64_t* __restrict__ rp,
                                                          const int* __restrict__ ci, const S* __restrict__ cv,
                                                          A* __restrict__ y) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  A* yt = reinterpret_cast<A*>(smem_raw);
  int* srp = reinterpret_cast<int*>(smem_raw + ((sizeof(A) * (size_t)m + 15) / 16) * 16);
  int* slp = srp + (m + 1);
  int* srw = slp + (nlev + 1);
  __shared__ A part[RUN_WARPS];
  const int64_t base = rp[0];
  for (int t = threadIdx.x; t < m; t += RUN_TPB) {
    yt[t] = y[s_tail + t];
    if (rows) srw[t] = rows[t];
  }
  for (int t = threadIdx.x; t <= m; t += RUN_TPB) srp[t] = (int)(rp[t] - base);
  for (int t = threadIdx.x; t <= nlev; t += RUN_TPB) slp[t] = lptr[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this warp's row r, entry range [q0, q1) with stride `step` in level l
  auto assign = [&](int l, int& r, int& q0, int& q1, int& step, int& G, int& slot, int& sub) {
    const int lo = slp[l], R = slp[l + 1] - lo;
    if (R >= RUN_WARPS) {
      G = 1;
      slot = warp;
      sub = 0;
    } else {
      G = RUN_WARPS / R;
      G = 1 << (31 - __clz(G));
      slot = warp / G;
      sub = warp % G;
    }
    step = 32 * G;
    if (slot < R) {
      const int t = lo + slot;
      r = rows ? srw[t] : t;
      q0 = srp[r] + sub * 32 + lane;
      q1 = srp[r + 1];
    } else {
      r = -1;
      q0 = q1 = 0;
    }
  };
  int r = -1, q0 = 0, q1 = 0, step = 32, G = 1, slot = 0, sub = 0;
  int pci = 0;
  A pcv = A(0);
  if (nlev > 0) {
    assign(0, r, q0, q1, step, G, slot, sub);
    if (q0 < q1) {
      pci = ci[base + q0];
      pcv = lda<A>(cv + base + q0);
    }
  }
  for (int l = 0; l < nlev; ++l) {
    const int lo = slp[l], hi = slp[l + 1], R = hi - lo;
    A acc = A(0);
    if (q0 < q1) {
      acc = pcv * yt[pci];
      for (int q = q0 + step; q < q1; q += step) acc = fma_(lda<A>(cv + base + q), yt[ci[base + q]], acc);
    }
    acc = wsum(acc);
    if (R >= RUN_WARPS) {
      if (lane == 0 && r >= 0) yt[r] = yt[r] - acc;
      for (int t = lo + warp + RUN_WARPS; t < hi; t += RUN_WARPS) {  // further rows of this warp
        const int rr = rows ? srw[t] : t;
        A a2 = A(0);
        for (int q = srp[rr] + lane; q < srp[rr + 1]; q += 32) a2 = fma_(lda<A>(cv + base + q), yt[ci[base + q]], a2);
        a2 = wsum(a2);
        if (lane == 0) yt[rr] = yt[rr] - a2;
      }
    } else if (lane == 0) {
      part[warp] = acc;
    }
    int nr = -1, nq0 = 0, nq1 = 0, nstep = 32, nG = 1, nslot = 0, nsub = 0;
    if (l + 1 < nlev) {  // prefetch the first entry of the next level
      assign(l + 1, nr, nq0, nq1, nstep, nG, nslot, nsub);
      if (nq0 < nq1) {
        pci = ci[base + nq0];
        pcv = lda<A>(cv + base + nq0);
      }
    }
    __syncthreads();
    if (R < RUN_WARPS) {
      if (slot < R && sub == 0 && lane == 0) {
        A t = part[warp];
        for (int j = 1; j < G; ++j) t = t + part[warp + j];
        yt[r] = yt[r] - t;
      }
      __syncthreads();
    }
    r = nr; q0 = nq0; q1 = nq1; step = nstep; G = nG; slot = nslot; sub = nsub;
  }
  for (int t = threadIdx.x; t < m; t += RUN_TPB) y[s_tail + t] = yt[t];
}

constexpr int TRI_TPB = 256;  // threads per CTA of the tile kernel

// Dense block product y = T x over a set of 64 x 64 tiles (column-major
// inside a tile), with the reduction inside a thread-block cluster: the CL
// CTAs of a cluster (8, or 16 where the GPU allows that non-portable size)
// share one tile row and each streams a contiguous chunk of its tiles
// (16-byte vectors of V consecutive rows of one tile column per thread;
// per-column partial sums added in a fixed order) into a 64-vector in its
// shared memory.  Rank 0 adds the CL vectors in rank order through
// distributed shared memory and writes the row, so results do not depend on
// timing.  x must not alias y.  The cluster size is a launch attribute
// (launch_tri), never left to a default.
// 16-byte read-only load of data read once per launch (tiles): issued as
// written, kept in its registers (no re-load at the point of use), no L1 allocation
__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}
template <class S, class A, int CL>
__global__ void __launch_bounds__(TRI_TPB)
    tri_cluster_kernel(const int4* __restrict__ items, const S* __restrict__ tiles, const A* __restrict__ x, int m,
                       A* __restrict__ y) {
  pdl_launch();
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  constexpr int V = 16 / sizeof(S);
  constexpr int RG = 64 / V;
  constexpr int CPS = TRI_TPB / RG;
  constexpr int NS = 64 / CPS;
  __shared__ A red[CPS][64];
  __shared__ A mine[64];
  const int4 it = items[blockIdx.x];
  const int cnt = it.z;
  const int rg = threadIdx.x % RG, cs = threadIdx.x / RG;
  A acc[V];
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = A(0);
  const uint4* tp = reinterpret_cast<const uint4*>(tiles) + (size_t)it.y * (64 * 64 / V);
  auto load = [&](int k, uint4* buf) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) buf[sl] = ld_stream(tp + (size_t)k * (64 * 64 / V) + (sl * CPS + cs) * RG + rg);
  };
  auto use = [&](int k, const uint4* buf) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) {
      const int c = (it.w + k) * 64 + sl * CPS + cs;
      const A xv = c < m ? x[c] : A(0);
      const S* e = reinterpret_cast<const S*>(&buf[sl]);
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] = fma_(lda<A>(e + v), xv, acc[v]);
    }
  };
  // One tile per step.  Measured on GB300 (fp32 factor, Anderson model,
  // ms per application): 40^3 0.220 -> 0.198 with these loads instead of
  // __ldg, 50^3 unchanged; issuing the next tile's loads before the current
  // tile's products made 50^3 slower (0.387 -> 0.410).
  // the first tile is read, and the others requested into L2, while the
  // predecessor (which writes x) finishes
  uint4 b0[NS];
  if (cnt > 1 && threadIdx.x == 0) l2_prefetch(tp + 64 * 64 / V, sizeof(S) * 64 * 64 * (size_t)(cnt - 1));
  if (cnt > 0) load(0, b0);
  pdl_wait();
  for (int k = 0; k < cnt; ++k) {
    if (k > 0) load(k, b0);
    use(k, b0);
  }
#pragma unroll
  for (int v = 0; v < V; ++v) red[cs][V * rg + v] = acc[v];
  __syncthreads();
  if (threadIdx.x < 64) {
    A sum = red[0][threadIdx.x];
#pragma unroll
    for (int j = 1; j < CPS; ++j) sum = sum + red[j][threadIdx.x];
    mine[threadIdx.x] = sum;
  }
  cl.sync();
  if (cl.block_rank() == 0 && threadIdx.x < 64) {
    A sum = A(0);
#pragma unroll
    for (int r = 0; r < CL; ++r) sum = sum + *cl.map_shared_rank(&mine[threadIdx.x], r);
    const int e = it.x * 64 + threadIdx.x;
    if (e < m) y[e] = sum;
  }
  cl.sync();  // the other ranks' shared memory stays alive until rank 0 has read it
}

// one launch of a cluster kernel: cl CTAs per cluster, PDL as launch_k
template <class... Params, class... Args>
static void launch_cl(void (*kern)(Params...), dim3 grid, dim3 block, int cl, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl ? 2 : 1;
  CK(cudaLaunchKernelEx(&cfg, kern, static_cast<Params>(args)...));
}
// items are grid-sized multiples of the cluster size (make_cluster_items)
template <class S, class A>
static void launch_tri(int items, int cl, const int4* it, const S* tiles, const A* x, int m, A* y, cudaStream_t s) {
  if (cl == 16) launch_cl(tri_cluster_kernel<S, A, 16>, dim3(items), dim3(TRI_TPB), 16, s, it, tiles, x, m, y);
  else launch_cl(tri_cluster_kernel<S, A, 8>, dim3(items), dim3(TRI_TPB), 8, s, it, tiles, x, m, y);
}
// Whether clusters of 16 tile CTAs can run on the current device: allows the
// non-portable size on both instantiations' kernel and asks the occupancy
// calculator for at least one active cluster.  Called on upload, before any
// graph capture.
template <class S, class A> bool tri_cluster16_ok() {
  auto kern = tri_cluster_kernel<S, A, 16>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16);
  cfg.blockDim = dim3(TRI_TPB);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 16;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int nc = 0;
  if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return nc > 0;
}

// raise the dynamic shared-memory limit of the tail kernel once per size
// (done before any graph capture: ildl_apply_graph calls it first)
template <class S, class A> static void ensure_tail_smem(size_t bytes) {
  // the attribute applies to the current device only: one raised size per device
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static size_t set[kMaxDev] = {};
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = set[dev < kMaxDev ? dev : kMaxDev - 1];
  if (dev >= kMaxDev || bytes > std::max<size_t>(cur, 48 * 1024)) {
    CK(cudaFuncSetAttribute(tail_run_kernel<S, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = std::max(cur, bytes);
  }
}

constexpr int kRunRows = 2 * RUN_WARPS;
constexpr int64_t kRunEntries = 16384;
template <class S>
void ildl_plan(DevFactor<S>& F, const std::vector<int64_t>& lp, const std::vector<int64_t>& up,
               const std::vector<int>& brows) {
  auto plan = [&](const std::vector<int>& ptr, bool fwd, std::vector<int>& seg) {
    seg.clear();
    const int nl = (int)ptr.size() - 1;
    int l = 1;  // level 0 has no off-diagonal entries in either sweep
    while (l < nl) {
      auto work = [&](int lv) {
        int64_t nz = 0;
        for (int t = ptr[lv]; t < ptr[lv + 1]; ++t) {
          int s = fwd ? t : brows[t];
          nz += fwd ? (lp[s + 1] - lp[s]) : (up[s + 1] - up[s]);
        }
        return nz;
      };
      // a level goes to the single-CTA run when each of its 32 warps has at
      // most two rows (one dependent load round each); wider levels are one
      // grid launch, whose cost does not grow with the row count
      int rows = ptr[l + 1] - ptr[l];
      int64_t nz = work(l);
      bool narrow = rows <= kRunRows && nz <= kRunEntries;
      if (!narrow) {
        seg.insert(seg.end(), {l, l + 1, lanes_for((double)nz / std::max(1, rows))});
        ++l;
        continue;
      }
      int l1 = l + 1;
      while (l1 < nl) {
        int r = ptr[l1 + 1] - ptr[l1];
        if (r > kRunRows || work(l1) > kRunEntries) break;
        ++l1;
      }
      seg.insert(seg.end(), {l, l1, 1});
      l = l1;
    }
  };
  plan(F.fptr, true, F.fseg);
  plan(F.bptr, false, F.bseg);
}
// levels of the bulk backward sweep start at 0 (rows may point into the tail)
template <class S> void ildl_plan_bwd0(DevFactor<S>& F, const std::vector<int64_t>& up, const std::vector<int>& brows) {
  std::vector<int> seg;
  for (size_t q = 0; q < F.bseg.size(); q += 3) seg.insert(seg.end(), {F.bseg[q], F.bseg[q + 1], F.bseg[q + 2]});
  if (F.bptr.size() > 1 && (F.bseg.empty() || F.bseg[0] != 0)) {
    int64_t nz = 0;
    for (int t = F.bptr[0]; t < F.bptr[1]; ++t) nz += up[brows[t] + 1] - up[brows[t]];
    std::vector<int> s0 = {0, 1, lanes_for((double)nz / std::max(1, F.bptr[1] - F.bptr[0]))};
    s0.insert(s0.end(), seg.begin(), seg.end());
    seg = s0;
  }
  F.bseg = seg;
}

// Coupling blocks of the multilevel form (symAMGsol.c:173-330 applies them
// with CSRMATVEC / CSRMATTVEC): the m rows of a CSR block (row pointers rp[t],
// t < m, global columns) written to y[r0 + t], LANES lanes per row, in the
// outer precision T.  SUB: y[r0 + t] -= sum_q v_q x[c_q]; else
// y[r0 + t] = sum_q v_q x[c_q].  The rows written and the columns read are
// disjoint ranges, so x may alias y.
template <class T, class S, int LANES, bool SUB>
__global__ void __launch_bounds__(WIDE_TPB) couple_kernel(int r0, int m, const int64_t* __restrict__ rp,
                                                         const int* __restrict__ ci, const S* __restrict__ cv,
                                                         const T* x, T* y) {
  pdl_begin();
  const int t = blockIdx.x * (WIDE_TPB / LANES) + (threadIdx.x / LANES);
  const int lane = threadIdx.x % LANES;
  const int r = r0 + t;
  T acc = T(0);
  if (t < m)
    for (int64_t q = rp[t] + lane; q < rp[t + 1]; q += LANES) acc = fma_(cvt<T>(ld_arith(cv + q)), x[ci[q]], acc);
  for (int o = LANES / 2; o > 0; o >>= 1) acc = acc + shfl_xor_any(acc, o);
  if (t < m && lane == 0) y[r] = SUB ? y[r] - acc : acc;
}
template <class T, class S, bool SUB>
static void launch_couple(int lanes, int r0, int m, const int64_t* rp, const int* ci, const S* cv, const T* x, T* y,
                          cudaStream_t s) {
  if (m <= 0) return;
  const int nb = m * lanes / WIDE_TPB + 1;
  if (lanes == 32) launch_k(couple_kernel<T, S, 32, SUB>, dim3(nb), dim3(WIDE_TPB), 0, s, r0, m, rp, ci, cv, x, y);
  else if (lanes == 16) launch_k(couple_kernel<T, S, 16, SUB>, dim3(nb), dim3(WIDE_TPB), 0, s, r0, m, rp, ci, cv, x, y);
  else launch_k(couple_kernel<T, S, 8, SUB>, dim3(nb), dim3(WIDE_TPB), 0, s, r0, m, rp, ci, cv, x, y);
}
// y[r] = yb[r] - t[r] for r in [r0, r0 + m)
template <class T>
__global__ void couple_combine_kernel(int r0, int m, const T* __restrict__ yb, const T* __restrict__ t, T* __restrict__ y) {
  pdl_begin();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) y[r0 + i] = yb[r0 + i] - t[r0 + i];
}

template <class T, class S> void ildl_apply(const DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s);

// The multilevel application with coupling blocks: per level l with rows B
// (steps [a, e)) and the later rows C,
//   forward:  y_B = B^{-1} y_B (the level's sub-factor), keep it, y_C -= F^H y_B;
//   backward: t_B = B^{-1} (F y_C), y_B = kept y_B - t_B.
template <class T, class S>
static void ildl_apply_coupled(const DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s) {
  const int n = F.n;
  const int nl = (int)F.lev.size();
  T* y = (T*)F.cy;
  T* yb = (T*)F.cyb;
  T* t = (T*)F.ct;
  launch_k(ildl_gather_kernel<T, T>, dim3(nblk(n)), dim3(TPB), 0, s, n, F.perm, b, y);
  for (int l = 0; l < nl; ++l) {
    const int a = F.lstart[l], e = F.lstart[l + 1];
    ildl_apply<T, S>(F.lev[l], spd, y + a, y + a, s);
    if (l + 1 < nl) {
      CK(cudaMemcpyAsync(yb + a, y + a, sizeof(T) * (size_t)(e - a), cudaMemcpyDeviceToDevice, s));
      launch_couple<T, S, true>(F.fh_lanes[l], e, n - e, F.fhp + F.fh_row0[l], F.fhi, F.fhx, y, y, s);
    }
  }
  for (int l = nl - 2; l >= 0; --l) {
    const int a = F.lstart[l], e = F.lstart[l + 1];
    launch_couple<T, S, false>(F.fp_lanes[l], a, e - a, F.fpp + a, F.fpi, F.fpx, y, t, s);
    ildl_apply<T, S>(F.lev[l], spd, t + a, t + a, s);
    launch_k(couple_combine_kernel<T>, dim3(nblk(e - a)), dim3(TPB), 0, s, a, e - a, (const T*)yb, (const T*)t, y);
  }
  launch_k(ildl_scatter_kernel<T, T>, dim3(nblk(n)), dim3(TPB), 0, s, n, F.perm, (const T*)y, x);
}

template <class T, class S> void ildl_apply(const DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s) {
  using A = typename Arith<S>::type;
  const int n = F.n;
  if (F.coupled) {
    ildl_apply_coupled<T, S>(F, spd, b, x, s);
    return;
  }
  launch_k(ildl_gather_kernel<T, A>, dim3(nblk(n)), dim3(TPB), 0, s, n, F.orig, b, F.y);
  auto sweep = [&](const std::vector<int>& seg, const std::vector<int>& ptr, const int* dptr, const int* rows,
                   const int64_t* rp, const int* ci, const S* cv) {
    for (size_t q = 0; q < seg.size(); q += 3) {
      int l0 = seg[q], l1 = seg[q + 1];
      if (seg[q + 2] == 1) {
        launch_k(ildl_run_kernel<S, A>, dim3(1), dim3(RUN_TPB), 0, s, l0, l1, dptr, rows, rp, ci, cv, F.y);
      } else {
        launch_wide<S, A>(seg[q + 2], ptr[l0], ptr[l0 + 1], rows, rp, ci, cv, F.y, s);
      }
    }
  };
  sweep(F.fseg, F.fptr, F.dfptr, nullptr, F.lp, F.li, F.lx);
  const bool dense = !F.blocks.empty(), levels = F.m_tail > 0 && !dense;
  auto ext = [&](int m, int s0, const int64_t* rp, const int* ci, const S* cv, int64_t entries, A* out) {
    launch_ext<S, A>(lanes_for((double)entries / std::max(1, m)), m, s0, rp, ci, cv, F.y, out, entries, s);
  };
  const size_t tsm = levels ? std::max(tail_smem_bytes<A>(F.m_tail, (int)F.tfptr.size() - 1, false),
                                       tail_smem_bytes<A>(F.m_tail, (int)F.tbptr.size() - 1, true))
                            : 0;
  if (levels) ensure_tail_smem<S, A>(tsm);
  if (dense) {
    for (const auto& B : F.blocks) {
      A* yb = F.y + B.s0;
      if (B.nt > 0) {
        // right-hand side into xb, then y_B = T xb
        ext(B.m, B.s0, B.ep, B.ei, B.ev, B.nfe, F.xb);
        launch_tri<S, A>(B.nitf, B.tcl, (const int4*)B.itf, B.tf, (const A*)F.xb, B.m, yb, s);
      } else if (B.nfe > 0) {
        ext(B.m, B.s0, B.ep, B.ei, B.ev, B.nfe, yb);
      }
    }
  } else if (levels) {
    ext(F.m_tail, F.s_tail, F.tep, F.tei, F.tev, 8 * (int64_t)F.m_tail, F.y + F.s_tail);
    launch_k(tail_run_kernel<S, A>, dim3(1), dim3(RUN_TPB), tsm, s, F.m_tail, F.s_tail, (int)F.tfptr.size() - 1, F.dtfptr, nullptr,
                                                 F.tip, F.tii, F.tiv, F.y);
  }
  launch_k(ildl_dsolve_kernel<S, A>, dim3(nblk(n)), dim3(TPB), 0, s, n, F.blk, F.partner, spd ? F.av : F.dv, spd ? F.aof : F.dof, F.y);
  if (dense) {
    for (auto it = F.blocks.rbegin(); it != F.blocks.rend(); ++it) {
      const auto& B = *it;
      A* yb = F.y + B.s0;
      if (B.nt > 0) {
        ext(B.m, B.s0, B.bp, B.bi, B.bv, B.nbe, F.xb);
        launch_tri<S, A>(B.nitb, B.tcl, (const int4*)B.itb, B.tb, (const A*)F.xb, B.m, yb, s);
      } else if (B.nbe > 0) {
        ext(B.m, B.s0, B.bp, B.bi, B.bv, B.nbe, yb);
      }
    }
  } else if (levels) {
    launch_k(tail_run_kernel<S, A>, dim3(1), dim3(RUN_TPB), tsm, s, F.m_tail, F.s_tail, (int)F.tbptr.size() - 1, F.dtbptr, F.tbrows,
                                                 F.tbp, F.tbi, F.tbv, F.y);
  }
  sweep(F.bseg, F.bptr, F.dbptr, F.brows, F.up, F.ui, F.ux);
  launch_k(ildl_scatter_kernel<T, A>, dim3(nblk(n)), dim3(TPB), 0, s, n, F.orig, F.y, x);
}

template <class T, class S> void ildl_apply_graph(DevFactor<S>& F, bool spd, const T* b, T* x, cudaStream_t s) {
  const int n = F.n;
  const int g = spd ? 1 : 0;
  if (!F.graph[g]) {
    using A = typename Arith<S>::type;
    auto smem = [](const DevFactor<S>& D) {
      if (D.m_tail > 0 && D.blocks.empty())
        ensure_tail_smem<S, A>(std::max(tail_smem_bytes<A>(D.m_tail, (int)D.tfptr.size() - 1, false),
                                        tail_smem_bytes<A>(D.m_tail, (int)D.tbptr.size() - 1, true)));
    };
    smem(F);
    for (const auto& D : F.lev) smem(D);
    cudaGraph_t gr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    ildl_apply<T, S>(F, spd, (const T*)F.rhs_in, (T*)F.sol_out, s);
    CK(cudaStreamEndCapture(s, &gr));
    size_t nn = 0;
    CK(cudaGraphGetNodes(gr, nullptr, &nn));
    F.graph_kernels[g] = (long long)nn;
    CK(cudaGraphInstantiate(&F.graph[g], gr, 0));
    CK(cudaGraphDestroy(gr));
  }
  if ((const void*)b != F.rhs_in) CK(cudaMemcpyAsync(F.rhs_in, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
  CK(cudaGraphLaunch(F.graph[g], s));
  g_launches += F.graph_kernels[g];
  if ((void*)x != F.sol_out) CK(cudaMemcpyAsync(x, F.sol_out, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
}

// ------------------------------------------------------- instantiations ----
#define JD_INST_T(T)                                                                               \
  template void spmv<T>(const SellMatrix<T>&, const T*, T*, cudaStream_t);                         \
  template void axpy<T>(long, T, const T*, T*, cudaStream_t);                                      \
  template void axpy_ratio<T>(long, const T*, const T*, double, const T*, T*, cudaStream_t);        \
  template void axpy_ratio_copy<T>(long, const T*, const T*, const T*, T*, T*, cudaStream_t);        \
  template void smooth<T>(long, T, const T*, double, T*, T*, cudaStream_t);                         \
  template void spmv_shift<T>(const SellMatrix<T>&, T, const T*, T*, cudaStream_t);                 \
  template void scal<T>(long, double, T*, cudaStream_t);                                           \
  template void fill<T>(long, T, T*, cudaStream_t);                                                \
  template void mdot<T>(long, int, const T*, long, const T*, T*, T*, cudaStream_t);                \
  template void gemv_dev<T>(long, int, T, const T*, long, const T*, T, T*, cudaStream_t);          \
  template void gemv_val<T>(long, int, T, const T*, long, const T*, T, T*, cudaStream_t);          \
  template void rmult<T>(long, int, int, const T*, long, const T*, T*, cudaStream_t);              \
  template void diagsolve<T>(long, const double*, const T*, T*, cudaStream_t);
JD_INST_T(double)
JD_INST_T(zc)
#define JD_INST_F(T, S)                                                                          \
  template void ildl_apply<T, S>(const DevFactor<S>&, bool, const T*, T*, cudaStream_t);          \
  template void ildl_apply_graph<T, S>(DevFactor<S>&, bool, const T*, T*, cudaStream_t);          \
  template void ildl_plan<S>(DevFactor<S>&, const std::vector<int64_t>&, const std::vector<int64_t>&, \
                             const std::vector<int>&);                                          \
  template void ildl_plan_bwd0<S>(DevFactor<S>&, const std::vector<int64_t>&, const std::vector<int>&); \
  template bool tri_cluster16_ok<S, typename Arith<S>::type>();
JD_INST_F(double, double)
JD_INST_F(double, float)
JD_INST_F(double, __nv_bfloat16)
JD_INST_F(zc, zc)
JD_INST_F(zc, cc)
JD_INST_F(zc, bc)

}  // namespace k
}  // namespace jdg
