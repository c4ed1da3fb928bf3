// tc_tiles.h -- the tile set and tile order of the tensor-core update (k_tc_gemm in
// tc_gemm.cu), host and device: the host counts the tiles, every CTA of the persistent kernel
// maps its tile indices to tiles, and the CPU tests check that the order visits every tile of
// the update region exactly once.
//
// The update region is one or two rectangles of C' (real rows x complex columns) that share
// the operands: rectangle r covers the first m_rows[r] rows of A' and the n_cols[r] columns of
// B' from b_col[r], and is written at (c_row0, c_col0[r]).  Tiles are TC_TM real rows x TC_TN
// columns.  Tiles of rectangle 0 come first; within a rectangle, groups of four row tiles, each
// whole group column by column (the CTAs at work share each B' tile four ways and the group's
// four A' row tiles across the wave), a partial last group row by row.
// lower = 1 (one square rectangle on the diagonal, symmetric updates): only the tiles that hold
// an element on or below the diagonal, i.e. column tile n <= m / 4 for row tile m (128 real rows
// = 64 complex rows against 256 columns); group g (row tiles 4g .. 4g+3) has g + 1 tiles per
// row and starts at tile 2 g (g + 1), so the group of a tile index is found in closed form.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define TT_HD __host__ __device__ __forceinline__
#else
#define TT_HD inline
#endif

constexpr int TC_TM = 128, TC_TN = 256;  // tile: real rows of C' x complex columns
constexpr int TC_CCH = 32;               // epilogue chunk: columns per reduce-add

struct TcRegion {
  int m_rows[2], n_cols[2], b_col[2], c_col0[2];
  int c_row0;
  int ntn[2], ntiles0, ntiles;
  int lower;
};

// the tile counts of a region whose m_rows, n_cols and lower are set
TT_HD void tc_region_count(TcRegion& Rg) {
  int ntl[2];
  for (int r = 0; r < 2; ++r) {
    Rg.ntn[r] = (Rg.n_cols[r] + TC_TN - 1) / TC_TN;
    if (Rg.ntn[r] < 1) Rg.ntn[r] = 1;
    const int ntm = (Rg.m_rows[r] + TC_TM - 1) / TC_TM;
    ntl[r] = (Rg.m_rows[r] > 0 && Rg.n_cols[r] > 0) ? Rg.ntn[r] * ntm : 0;
  }
  Rg.ntiles0 = ntl[0];
  Rg.ntiles = ntl[0] + ntl[1];
  if (Rg.lower) {  // tiles n <= m / 4 of every row tile m
    const int ntm = (Rg.m_rows[0] + TC_TM - 1) / TC_TM;
    long long cnt = 0;
    for (int m = 0; m < ntm; ++m) cnt += (m / 4 + 1 < Rg.ntn[0]) ? m / 4 + 1 : Rg.ntn[0];
    Rg.ntiles0 = Rg.ntiles = (int)cnt;
  }
}

// tile index -> (rectangle r, first real row m0, first column n0 within the rectangle); false:
// the tile lies beyond its rectangle (an index of a partial last group past its rows)
TT_HD bool tc_tile_at(const TcRegion& Rg, int tile, int& r, int& m0, int& n0) {
  if (Rg.lower) {
    r = 0;
    int g = (int)((sqrtf(2.f * (float)tile + 1.f) - 1.f) * 0.5f);
    while (2 * g * (g + 1) > tile) --g;
    while (2 * (g + 1) * (g + 2) <= tile) ++g;
    const int t = tile - 2 * g * (g + 1);
    if (4 * (g + 1) * TC_TM <= Rg.m_rows[0]) {
      m0 = (4 * g + (t & 3)) * TC_TM;
      n0 = (t >> 2) * TC_TN;
    } else {
      m0 = (4 * g + t / (g + 1)) * TC_TM;
      n0 = (t % (g + 1)) * TC_TN;
    }
    return m0 < Rg.m_rows[0];
  }
  r = tile < Rg.ntiles0 ? 0 : 1;
  const int lt = r ? tile - Rg.ntiles0 : tile;
  const int ntn = Rg.ntn[r], G = lt / (4 * ntn), l = lt - G * 4 * ntn;
  if (4 * (G + 1) * TC_TM <= Rg.m_rows[r]) {
    m0 = (4 * G + (l & 3)) * TC_TM;
    n0 = (l >> 2) * TC_TN;
  } else {
    m0 = (4 * G + l / ntn) * TC_TM;
    n0 = (l % ntn) * TC_TN;
  }
  return m0 < Rg.m_rows[r];
}

// epilogue chunks of a tile that hold a column of its rectangle (n0 < n_cols): the rest of the
// accumulator is not read, its reduce-adds would lie wholly outside the tensor map
TT_HD int tc_tile_chunks(int n_cols, int n0) {
  const int c = (n_cols - n0 + TC_CCH - 1) / TC_CCH;
  return c < 1 ? 1 : (c > TC_TN / TC_CCH ? TC_TN / TC_CCH : c);
}
