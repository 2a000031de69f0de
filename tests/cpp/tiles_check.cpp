// Checks the tile-list builders of the tensor-core pair kernels
// (cpptraj_gb300/csrc/gbr_tiles.h) against a direct restatement: every tile of
// the grouped order with a pair in the output region, then a stable
// partition by the first input chunk that covers the frames the tile reads.
#include <cstdio>
#include <random>
#include <vector>

#include "gbr_tiles.h"

using gbr::TileGrid;

static std::vector<int2> direct_grouped(const TileGrid& g) {
  std::vector<int2> out;
  const int64_t Ti = (g.i_end - g.i_base + g.rows - 1) / g.rows, Tj = (g.jt_end - g.jt_base + g.cols - 1) / g.cols;
  for (int64_t g0 = 0; g0 < Ti; g0 += 8)
    for (int64_t tj = 0; tj < Tj; ++tj)
      for (int64_t ti = g0; ti < std::min(Ti, g0 + 8); ++ti) {
        if (g.tri && g.jt_base + tj * g.cols + g.cols - 1 <= g.i_base + ti * g.rows) continue;
        out.push_back(gbr::tile2(ti, tj));
      }
  return out;
}

int main() {
  std::mt19937_64 rng(20240611);
  const int64_t rows_opts[4] = {42, 84, 80, 40};
  int bad = 0;
  for (int it = 0; it < 20000; ++it) {
    const int64_t n = 1 + (int64_t)(rng() % 3000);
    const int64_t rb = (int64_t)(rng() % n);
    const int64_t re = rb + (int64_t)(rng() % (n - rb + 1));
    const int64_t rows = rows_opts[rng() % 4];
    const bool tri = rng() % 4 != 0;
    const TileGrid g = tri ? TileGrid{rb, re, rb, n, rows, 64, true} : TileGrid{0, n, rb, re, rows, 64, false};
    const int nch = 1 + (int)(rng() % 8);
    int64_t ce[8];
    for (int c = 0; c < nch; ++c) ce[c] = n * (c + 1) / nch;

    const std::vector<int2> grouped = direct_grouped(g);
    std::vector<int2> built;
    const int64_t nt = gbr::build_tiles_grouped(g, built);
    bool ok = nt == (int64_t)grouped.size();
    for (int64_t t = 0; ok && t < nt; ++t) ok = built[t].x == grouped[t].x && built[t].y == grouped[t].y;

    std::vector<int> stage(grouped.size());
    std::vector<int64_t> off(nch + 1, 0);
    for (size_t t = 0; t < grouped.size(); ++t) {
      const int64_t fe = std::min(std::max(g.i_base + (grouped[t].x + 1) * rows, g.jt_base + (grouped[t].y + 1) * 64), n);
      int c = 0;
      while (c < nch - 1 && ce[c] < fe) ++c;
      stage[t] = c;
      off[c + 1]++;
    }
    for (int c = 0; c < nch; ++c) off[c + 1] += off[c];
    std::vector<int2> expect(grouped.size());
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (size_t t = 0; t < grouped.size(); ++t) expect[fill[stage[t]]++] = grouped[t];

    std::vector<int2> got(grouped.size() + 1);
    int64_t so[9];
    std::vector<int64_t> scratch;
    const int64_t n2 = gbr::build_tiles_staged(g, ce, nch, n, got.data(), nt, so, scratch);
    ok = ok && n2 == nt;
    for (int c = 0; ok && c <= nch; ++c) ok = so[c] == off[c];
    for (int64_t t = 0; ok && t < nt; ++t) ok = got[t].x == expect[t].x && got[t].y == expect[t].y;
    if (ok && nt > 0) ok = gbr::build_tiles_staged(g, ce, nch, n, got.data(), nt - 1, so, scratch) == -1;
    if (!ok && bad++ < 5)
      std::printf("mismatch: n=%lld rows=[%lld,%lld) tile_rows=%lld tri=%d chunks=%d\n", (long long)n, (long long)rb,
                  (long long)re, (long long)rows, (int)tri, nch);
  }
  std::printf("%s\n", bad ? "FAIL" : "OK");
  return bad ? 1 : 0;
}
