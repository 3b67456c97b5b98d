// Plan of the dense blocks of a factor's forward levels (host side, pure).
#pragma once
#include <cstdint>
#include <vector>

#include "tail_inverse.hpp"

namespace jdg {

// Blocks after the bulk levels.  Each group {a, b, dense} covers forward
// levels [a, b); dense groups are solved with the explicit inverse of their
// diagonal block, the others are single levels.  The plan minimises a model
// of one application (both sweeps) over the split point between the bulk
// (levels [0, first)) and the blocks:
//   - a bulk level costs t_bulk per sweep (one launch each with the level
//     kernels; one dependency step of the single sync-free sweep kernel)
//     plus its entries' bytes;
//   - a single-level block costs one launch per sweep plus its bytes;
//   - a dense block is charged three launches per sweep plus its external
//     entries and both tile sets.
// Shallow factors keep the level path entirely (empty plan): below a saving
// of min_saving per application, building and uploading the tiles costs
// more than a solve gains, and substitution order keeps the rounding of the
// sequential algorithm.
struct BlockGroup {
  int a, b;
  bool dense;
};
inline std::vector<BlockGroup> plan_dense_blocks(const std::vector<int>& fptr, const std::vector<int64_t>& ent_f,
                                                 const std::vector<int64_t>& ent_b, size_t elem_bytes, int dense_max,
                                                 double min_saving, double t_bulk = 4e-6, double t_launch = 4e-6,
                                                 double bw = 5.0e12) {
  const int nfl = (int)fptr.size() - 1;
  const double eb = (double)elem_bytes + 4;
  auto bytes = [&](int l) { return (double)(ent_f[l] + ent_b[l]) * eb / bw; };
  // level 0 has no entries in the forward sweep: one launch (or step) less
  auto c_bulk = [&](int l) { return (l > 0 ? 2 : 1) * t_bulk + bytes(l); };
  auto c_single = [&](int l) { return (l > 0 ? 2 : 1) * t_launch + bytes(l); };
  // tail[a]: the cheapest cover of levels [a, nfl) by blocks
  std::vector<double> tail(nfl + 1, 0.0);
  std::vector<int> nxt(nfl + 1, -1);
  for (int a = nfl - 1; a >= 1; --a) {
    tail[a] = c_single(a) + tail[a + 1];
    double ent = 0;
    for (int b = a + 1; b <= nfl; ++b) {
      const int m = fptr[b] - fptr[a];
      if (m > dense_max) break;
      ent += (double)(ent_f[b - 1] + ent_b[b - 1]);
      const double nt = (m + kTile - 1) / kTile;
      const double c = 6 * t_launch + 2.0 * nt * (nt + 1) / 2 * kTileElems * elem_bytes / bw + ent * eb / bw;
      if (c + tail[b] < tail[a]) {
        tail[a] = c + tail[b];
        nxt[a] = b;
      }
    }
  }
  // the split: bulk levels [0, first), blocks from first on (first = nfl: no blocks)
  double bulk = 0, all_levels = 0;
  for (int l = 0; l < nfl; ++l) all_levels += c_bulk(l);
  double best = all_levels;
  int first = nfl;
  for (int a = 1; a < nfl; ++a) {
    bulk += c_bulk(a - 1);
    if (nxt[a] >= 0 && bulk + tail[a] < best) {  // a block plan starts with a dense group
      best = bulk + tail[a];
      first = a;
    }
  }
  std::vector<BlockGroup> g;
  if (first >= nfl || all_levels - best < min_saving) return g;
  for (int a = first; a < nfl;) {
    if (nxt[a] >= 0) {
      g.push_back({a, nxt[a], true});
      a = nxt[a];
    } else {
      g.push_back({a, a + 1, false});
      ++a;
    }
  }
  return g;
}

}  // namespace jdg
