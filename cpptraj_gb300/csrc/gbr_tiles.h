// Tile lists of the tensor-core pair kernels (host side).
//
// A launch tile covers `rows` reference frames × `cols` target frames of the
// output. Tiles are listed in grouped order: groups of 8 tile rows swept
// column by column, so the CTAs in flight share their reference and target
// frames in L2. For a triangle (TRI), tiles holding no pair with
// target > reference are left out.
#pragma once

#include <vector_types.h>

#include <algorithm>
#include <cstdint>
#include <vector>

namespace gbr {

struct TileGrid {
  int64_t i_base, i_end;    // reference frame range
  int64_t jt_base, jt_end;  // target frame range
  int64_t rows, cols;       // frames per launch tile
  bool tri;
};

constexpr int64_t kTileGroup = 8;

inline int2 tile2(int64_t ti, int64_t tj) {
  int2 v;
  v.x = (int)ti;
  v.y = (int)tj;
  return v;
}

// Calls run(g0, tj, te) for every (group, column) run of the grouped order:
// tiles (ti, tj) for ti in [g0, te). `col_end` is scratch.
template <class Run>
inline void for_each_tile_run(const TileGrid& g, std::vector<int64_t>& col_end, Run&& run) {
  const int64_t Ti = (g.i_end - g.i_base + g.rows - 1) / g.rows, Tj = (g.jt_end - g.jt_base + g.cols - 1) / g.cols;
  // TRI: a tile holds a pair with target > reference only while its first
  // reference frame i_base + ti * rows is below the tile's last target frame
  // jt_base + tj * cols + cols - 1: tile rows below col_end[tj].
  col_end.resize((size_t)std::max<int64_t>(Tj, 1));
  for (int64_t tj = 0; tj < Tj; ++tj) {
    const int64_t d = g.jt_base + tj * g.cols + g.cols - 1 - g.i_base;
    col_end[tj] = g.tri ? std::min(Ti, d > 0 ? (d + g.rows - 1) / g.rows : 0) : Ti;
  }
  for (int64_t g0 = 0; g0 < Ti; g0 += kTileGroup) {
    const int64_t ge = std::min(Ti, g0 + kTileGroup);
    for (int64_t tj = 0; tj < Tj; ++tj) {
      const int64_t te = std::min(ge, col_end[tj]);
      if (te > g0) run(g0, tj, te);
    }
  }
}

inline int64_t build_tiles_grouped(const TileGrid& g, std::vector<int2>& tiles) {
  std::vector<int64_t> col_end;
  tiles.clear();
  for_each_tile_run(g, col_end, [&](int64_t g0, int64_t tj, int64_t te) {
    for (int64_t ti = g0; ti < te; ++ti) tiles.push_back(tile2(ti, tj));
  });
  return (int64_t)tiles.size();
}

// The grouped list, stably partitioned by stage: the stage of a tile is the
// first of the n_chunks input chunks (frames [0, chunk_end[c])) that covers
// every frame the tile reads, i.e. the number of chunk ends below
// min(max(i_base + (ti + 1) * rows, jt_base + (tj + 1) * cols), F).
// stage_off[0..n_chunks] receives the stage offsets. Writes nothing and
// returns -1 if the list holds more than cap tiles or n_chunks is outside
// [1, 64]; else returns its length.
// Within a run the reference end grows with ti, so the tiles up to the one
// whose reference end passes the run's target end share the run's stage.
inline int64_t build_tiles_staged(const TileGrid& g, const int64_t* chunk_end, int n_chunks, int64_t F, int2* dst,
                                  int64_t cap, int64_t* stage_off, std::vector<int64_t>& scratch) {
  if (n_chunks < 1 || n_chunks > 64) return -1;
  const int64_t Ti = (g.i_end - g.i_base + g.rows - 1) / g.rows, Tj = (g.jt_end - g.jt_base + g.cols - 1) / g.cols;
  auto stage_of = [&](int64_t fe) {
    fe = std::min(fe, F);
    int64_t c = 0;
    for (int k = 0; k < n_chunks - 1; ++k) c += (chunk_end[k] < fe) ? 1 : 0;
    return c;
  };
  // Per tile row: the stage of its reference end. Per column: the stage of
  // its target end, and the tile rows (below col_mid) whose reference end is
  // at most that target end.
  scratch.resize((size_t)(std::max<int64_t>(Ti, 1) + 3 * std::max<int64_t>(Tj, 1)));
  int64_t* row_stage = scratch.data();
  int64_t* col_stage = row_stage + std::max<int64_t>(Ti, 1);
  int64_t* col_mid = col_stage + std::max<int64_t>(Tj, 1);
  std::vector<int64_t> col_end_v;
  for (int64_t ti = 0; ti < Ti; ++ti) row_stage[ti] = stage_of(g.i_base + (ti + 1) * g.rows);
  for (int64_t tj = 0; tj < Tj; ++tj) {
    const int64_t b = g.jt_base + (tj + 1) * g.cols;
    col_stage[tj] = stage_of(b);
    col_mid[tj] = b > g.i_base ? (b - g.i_base) / g.rows : 0;
  }
  for (int c = 0; c <= n_chunks; ++c) stage_off[c] = 0;
  int64_t* cnt = stage_off + 1;
  for_each_tile_run(g, col_end_v, [&](int64_t g0, int64_t tj, int64_t te) {
    const int64_t mid = std::min(std::max(col_mid[tj], g0), te);
    cnt[col_stage[tj]] += mid - g0;
    for (int64_t ti = mid; ti < te; ++ti) cnt[row_stage[ti]]++;
  });
  for (int c = 0; c < n_chunks; ++c) stage_off[c + 1] += stage_off[c];
  const int64_t nt = stage_off[n_chunks];
  if (nt > cap) return -1;
  int64_t fill[64];
  for (int c = 0; c < n_chunks; ++c) fill[c] = stage_off[c];
  for_each_tile_run(g, col_end_v, [&](int64_t g0, int64_t tj, int64_t te) {
    const int64_t mid = std::min(std::max(col_mid[tj], g0), te);
    int2* out = dst + fill[col_stage[tj]];
    for (int64_t ti = g0; ti < mid; ++ti) *out++ = tile2(ti, tj);
    fill[col_stage[tj]] += mid - g0;
    for (int64_t ti = mid; ti < te; ++ti) dst[fill[row_stage[ti]]++] = tile2(ti, tj);
  });
  return nt;
}

}  // namespace gbr
