// Symmetric scaling from a maximum-product perfect matching, host side.
//
// Plays the role of the reference's MC64 step (called with matching = 1 by
// src/jd/JDaux.F:741 through src/ilupack/symilupackfactor.c:184-193 and
// sympermMC64amd.c:282-284; HSL MC64 itself is not part of the reference).
// This is the project's own code for the published method (Duff and Koster,
// "On algorithms for permuting large entries to the diagonal of a sparse
// matrix", SIAM J. Matrix Anal. Appl. 22, 2001; symmetric use after Duff and
// Pralet, 2005):
//
//  * costs c_ij = log(max_k |a_kj|) - log|a_ij| >= 0 on the full pattern;
//  * a perfect matching of minimum total cost (= maximum product of the
//    matched |a_ij| relative to their column maxima) by successive shortest
//    augmenting paths (Dijkstra on reduced costs c_ij - u_i - v_j >= 0, the
//    duals updated after each augmentation so matched edges keep reduced
//    cost 0);
//  * row scale exp(u_i), column scale exp(v_j) / max_k |a_kj|: every scaled
//    entry has modulus exp(-(reduced cost)) <= 1, and 1 on the matching;
//  * symmetric scale d_i = sqrt(row_i * col_i).
//
// A structurally singular pattern has no perfect matching; the rows left
// unmatched get the scale 1 / sqrt(max |a_i.|) (or 1 for an empty row).
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <queue>
#include <utility>
#include <vector>

namespace jdg {

// Full symmetric pattern: for row i, columns cols[i][*] with moduli mods[i][*]
// (including the diagonal when it is nonzero).  Returns the symmetric scale;
// `matched` (optional) receives the number of matched rows and `partner`
// (optional) the matched column of each row (-1 when unmatched).
inline std::vector<double> matching_scale(int n, const std::vector<std::vector<int>>& cols,
                                          const std::vector<std::vector<double>>& mods, int* matched = nullptr,
                                          std::vector<int>* partner = nullptr) {
  const double inf = std::numeric_limits<double>::infinity();
  // the matrix is symmetric: column j's entries are row j's
  std::vector<double> cmax(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (double m : mods[j]) cmax[j] = std::max(cmax[j], m);
  // cost of entry (i, j), stored with row j's list (column j)
  auto cost = [&](int j, size_t q) { return std::log(cmax[j]) - std::log(mods[j][q]); };
  std::vector<double> u(n, 0.0), v(n, 0.0);
  std::vector<int> row_of_col(n, -1), col_of_row(n, -1);
  // initial duals and a greedy matching on zero reduced costs
  for (int j = 0; j < n; ++j) v[j] = 0.0;  // the column maximum has cost 0
  for (int i = 0; i < n; ++i) {  // u_i = min_j c_ij (entry (i, j) is row i's entry q, |a_ij| = mods[i][q])
    double m = inf;
    for (size_t q = 0; q < cols[i].size(); ++q)
      if (mods[i][q] > 0) m = std::min(m, std::log(cmax[cols[i][q]]) - std::log(mods[i][q]));
    u[i] = (m < inf) ? m : 0.0;
  }
  for (int j = 0; j < n; ++j)
    for (size_t q = 0; q < cols[j].size(); ++q) {
      const int i = cols[j][q];
      if (mods[j][q] <= 0 || col_of_row[i] >= 0) continue;
      if (cost(j, q) - u[i] - v[j] <= 0.0) {
        col_of_row[i] = j;
        row_of_col[j] = i;
        break;
      }
    }
  // successive shortest augmenting paths from the free columns
  std::vector<double> d(n, inf), dcol(n, inf);
  std::vector<int> pred(n, -1), done_rows, reached_rows;
  std::vector<char> final_row(n, 0);
  using Item = std::pair<double, int>;
  for (int j0 = 0; j0 < n; ++j0) {
    if (row_of_col[j0] >= 0) continue;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    done_rows.clear();
    reached_rows.clear();
    std::vector<int> final_cols{j0};
    dcol[j0] = 0.0;
    auto relax_from = [&](int j) {
      for (size_t q = 0; q < cols[j].size(); ++q) {
        if (mods[j][q] <= 0) continue;
        const int i = cols[j][q];
        if (final_row[i]) continue;
        const double nd = dcol[j] + (cost(j, q) - u[i] - v[j]);
        if (nd < d[i]) {
          if (d[i] == inf) reached_rows.push_back(i);
          d[i] = nd;
          pred[i] = j;
          heap.push({nd, i});
        }
      }
    };
    relax_from(j0);
    int free_row = -1;
    double L = inf;
    while (!heap.empty()) {
      auto [di, i] = heap.top();
      heap.pop();
      if (final_row[i] || di > d[i]) continue;
      final_row[i] = 1;
      done_rows.push_back(i);
      if (col_of_row[i] < 0) {
        free_row = i;
        L = di;
        break;
      }
      const int j = col_of_row[i];
      dcol[j] = di;
      final_cols.push_back(j);
      relax_from(j);
    }
    if (free_row >= 0) {
      // duals: finalized rows u += d - L, finalized columns v += L - dcol
      for (int i : done_rows) u[i] += d[i] - L;
      for (int j : final_cols) v[j] += L - dcol[j];
      // augment along the predecessor columns
      int i = free_row;
      for (;;) {
        const int j = pred[i];
        const int inext = row_of_col[j];
        row_of_col[j] = i;
        col_of_row[i] = j;
        if (j == j0) break;
        i = inext;
      }
    }
    for (int i : reached_rows) {
      d[i] = inf;
      final_row[i] = 0;
      pred[i] = -1;
    }
    for (int j : final_cols) dcol[j] = inf;
  }
  int nm = 0;
  std::vector<double> s(n, 1.0);
  for (int i = 0; i < n; ++i) {
    if (col_of_row[i] >= 0 && cmax[i] > 0) {
      ++nm;
      // row scale exp(u_i), column scale exp(v_i) / cmax_i
      s[i] = std::exp(0.5 * (u[i] + v[i])) / std::sqrt(cmax[i]);
    } else {
      s[i] = cmax[i] > 0 ? 1.0 / std::sqrt(cmax[i]) : 1.0;
    }
  }
  if (matched) *matched = nm;
  if (partner) *partner = col_of_row;
  return s;
}

}  // namespace jdg
