// Explicit inverse of the deepest part of the ILDL factor ("dense tail").
//
// The rows of the last forward levels form a unit lower-triangular block
// L_TT whose dependency chains are hundreds to thousands of levels deep but
// only a few rows wide.  Solving it level by level costs one dependent memory
// round trip per level; multiplying by its explicit inverse costs one pass
// over the inverse's bytes at full memory bandwidth.  This file computes the
// inverse on the host (in the host arithmetic, double or complex<double>) and
// lays it out as 64 x 64 tiles for the device kernels:
//   forward set : Linv, tile rows I = 0..nt-1 hold tile columns 0..I;
//   backward set: Linv^H (upper triangular), tile rows J hold columns J..nt-1.
// Each tile is stored column-major (element (r, c) at c*64 + r); entries past
// the block's size m are zero.
#pragma once
#include <algorithm>
#include <atomic>
#include <complex>
#include <cstdint>
#include <thread>
#include <vector>

namespace jdg {

constexpr int kTile = 64;
constexpr int kTileElems = kTile * kTile;

inline double conj_h(double v) { return v; }
inline std::complex<double> conj_h(const std::complex<double>& v) { return std::conj(v); }

inline int64_t lower_tile_offset(int I) { return (int64_t)I * (I + 1) / 2; }
inline int64_t upper_tile_offset(int J, int nt) { return (int64_t)J * nt - (int64_t)J * (J - 1) / 2; }

// Work items of the tile kernel, 4 ints each: {tile row, first tile (storage
// index), tile count, first tile column}.  Every tile row gets exactly
// `per_row` items (one thread-block cluster), each with a contiguous chunk of
// the row's tiles (some chunks may be empty); the item of cluster rank r of
// row i is item i * per_row + r.
inline std::vector<int> make_cluster_items(int nt, bool lower, int per_row) {
  std::vector<int> item;
  item.reserve((size_t)nt * per_row * 4);
  for (int i = 0; i < nt; ++i) {
    const int c0 = lower ? 0 : i, cnt = lower ? i + 1 : nt - i;
    const int64_t off = lower ? lower_tile_offset(i) : upper_tile_offset(i, nt);
    const int chunk = (cnt + per_row - 1) / per_row;
    for (int r = 0; r < per_row; ++r) {
      const int k0 = std::min(cnt, r * chunk), k1 = std::min(cnt, k0 + chunk);
      item.insert(item.end(), {i, (int)(off + k0), k1 - k0, c0 + k0});
    }
  }
  return item;
}

// rp/ci/cv: rows t = 0..m-1 of L_TT without the unit diagonal, columns local
// (ci < t).  Fills tf (forward) and tb (backward) with nt*(nt+1)/2 tiles each,
// converting with store(H) -> S.  Column blocks of 64 run on `threads` host
// threads; every block is computed the same way whatever the thread count.
template <class H, class S, class Store>
void tail_inverse(int m, const std::vector<int64_t>& rp, const std::vector<int>& ci, const std::vector<H>& cv,
                  std::vector<S>& tf, std::vector<S>& tb, int threads, Store store) {
  const int nt = (m + kTile - 1) / kTile;
  const int64_t ntiles = (int64_t)nt * (nt + 1) / 2;
  tf.assign((size_t)ntiles * kTileElems, store(H(0)));
  tb.assign((size_t)ntiles * kTileElems, store(H(0)));
  if (m == 0) return;
  std::atomic<int> next{0};
  auto worker = [&]() {
    std::vector<H> X;
    for (;;) {
      const int J = next.fetch_add(1);
      if (J >= nt) break;
      const int j0 = J * kTile;
      const int rows = m - j0;
      X.assign((size_t)rows * kTile, H(0));
      // columns j0..j0+63 of Linv by forward substitution: X row i - j0
      // holds Linv(i, j0 + c)
      for (int i = j0; i < m; ++i) {
        H* xi = X.data() + (size_t)(i - j0) * kTile;
        if (i < j0 + kTile) xi[i - j0] = H(1);
        for (int64_t q = rp[i]; q < rp[i + 1]; ++q) {
          const int c = ci[q];
          if (c < j0) continue;
          const H l = cv[q];
          const H* xc = X.data() + (size_t)(c - j0) * kTile;
          for (int k = 0; k < kTile; ++k) xi[k] -= l * xc[k];
        }
      }
      // scatter into the tiles (I, J), I >= J, and their adjoints (J, I)
      for (int I = J; I < nt; ++I) {
        S* ft = tf.data() + (size_t)(lower_tile_offset(I) + J) * kTileElems;
        S* bt = tb.data() + (size_t)(upper_tile_offset(J, nt) + (I - J)) * kTileElems;
        for (int r = 0; r < kTile; ++r) {
          const int i = I * kTile + r;
          if (i >= m) break;
          const H* xi = X.data() + (size_t)(i - j0) * kTile;
          for (int c = 0; c < kTile; ++c) {
            // forward tile element (r, c) = Linv(I*64 + r, J*64 + c)
            ft[(size_t)c * kTile + r] = store(xi[c]);
            // backward tile (J, I) element (c, r) = conj(Linv(I*64 + r, J*64 + c))
            bt[(size_t)r * kTile + c] = store(conj_h(xi[c]));
          }
        }
      }
    }
  };
  const int nth = std::max(1, std::min(threads, nt));
  std::vector<std::thread> pool;
  for (int t = 1; t < nth; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
}

}  // namespace jdg
