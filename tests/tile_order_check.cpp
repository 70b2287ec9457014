// Host check of crocodile_gb300/csrc/tile_order.h: for every block edge and
// a range of grid shapes, every tile number lies in [0, tpl), distinct tiles
// get distinct numbers, and tile_xy inverts tile_index.  Also prints the
// numbers of a few tiles for the Python replica in tests/test_tile_order_cpu.py.
// Exit status 0 when everything holds.
#include <cstdio>
#include <vector>

#include "tile_order.h"

using namespace cg;

int main() {
  long bad = 0, checked = 0;
  const int shapes[][2] = {{1, 1}, {1, 7}, {3, 5}, {12, 12}, {16, 16}, {22, 22}, {31, 33},
                           {86, 86}, {128, 128}, {171, 86}, {512, 512}, {513, 300}, {1024, 1}};
  for (auto &sh : shapes) {
    const int ntx = sh[0], nty = sh[1];
    const int tblog = tile_block_log(ntx, nty);
    const int B = 1 << tblog;
    const int nbx = (ntx + B - 1) / B, nby = (nty + B - 1) / B;
    const long tpl = (long)nbx * nby * B * B;
    std::vector<char> seen(tpl, 0);
    for (int ty = 0; ty < nty; ++ty)
      for (int tx = 0; tx < ntx; ++tx) {
        const int t = tile_index(tx, ty, tblog, nbx);
        ++checked;
        if (t < 0 || t >= tpl || seen[t]) {
          ++bad;
          continue;
        }
        seen[t] = 1;
        int x, y;
        tile_xy(t, tblog, nbx, x, y);
        if (x != tx || y != ty) ++bad;
      }
  }
  printf("tiles: %ld bad of %ld\n", bad, checked);
  // reference values: (ntx, nty, tx, ty) -> t
  const int probe[][4] = {{512, 512, 0, 0}, {512, 512, 1, 0}, {512, 512, 0, 1},
                          {512, 512, 31, 31}, {512, 512, 32, 0}, {512, 512, 0, 32},
                          {512, 512, 511, 511}, {86, 86, 85, 40}, {12, 12, 11, 5}};
  for (auto &q : probe)
    printf("probe %d %d %d %d %d\n", q[0], q[1], q[2], q[3],
           tile_index(q[2], q[3], tile_block_log(q[0], q[1]),
                      (q[0] + (1 << tile_block_log(q[0], q[1])) - 1) >>
                          tile_block_log(q[0], q[1])));
  return bad ? 1 : 0;
}
