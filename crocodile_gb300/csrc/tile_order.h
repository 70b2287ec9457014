// Tile numbering of the tiled plans (plain C++, also compiled for the host
// checks of tests/tile_order_check.cpp).
//
// The tiles of one grid layer are numbered along a Morton (Z-order) curve
// inside square blocks of 2^tblog x 2^tblog tiles (tblog <= 5), the blocks in
// row-major order, nbx blocks per row.  Work items follow tile numbers and
// the persistent gridders take them in that order, so the tiles in flight at
// any time lie close together and the kernel slices that nearby visibilities
// share are reused from L2 (tile rows in row-major order lie too far apart
// for that).
#pragma once

#ifdef __CUDACC__
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#endif

namespace cg {

CG_HD unsigned spread_bits(unsigned a) {  // low 8 bits -> even bits
  a &= 0xffu;
  a = (a | (a << 4)) & 0x0f0fu;
  a = (a | (a << 2)) & 0x3333u;
  return (a | (a << 1)) & 0x5555u;
}

CG_HD unsigned compact_bits(unsigned a) {  // even bits -> low 8 bits
  a &= 0x5555u;
  a = (a | (a >> 1)) & 0x3333u;
  a = (a | (a >> 2)) & 0x0f0fu;
  return (a | (a >> 4)) & 0x00ffu;
}

// Number of tile (tx, ty); in [0, nbx * nby * 4^tblog) for tx < nbx * 2^tblog,
// ty < nby * 2^tblog.
CG_HD int tile_index(int tx, int ty, int tblog, int nbx) {
  const int m = (1 << tblog) - 1;
  return ((((ty >> tblog) * nbx + (tx >> tblog)) << (2 * tblog)) |
          (int)(spread_bits((unsigned)(tx & m)) | (spread_bits((unsigned)(ty & m)) << 1)));
}

// Inverse of tile_index.
CG_HD void tile_xy(int t, int tblog, int nbx, int &tx, int &ty) {
  const int blk = t >> (2 * tblog);
  const unsigned m = (unsigned)t & ((1u << (2 * tblog)) - 1u);
  tx = ((blk % nbx) << tblog) | (int)compact_bits(m);
  ty = ((blk / nbx) << tblog) | (int)compact_bits(m >> 1);
}

// Block edge for a layer of ntx x nty tiles: the smallest power of two that
// covers it, at most 32 tiles.
CG_HD int tile_block_log(int ntx, int nty) {
  const int big = ntx > nty ? ntx : nty;
  int b = 0;
  while (b < 5 && (1 << b) < big) ++b;
  return b;
}

}  // namespace cg
