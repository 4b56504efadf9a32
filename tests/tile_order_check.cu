// Host check of the Gram kernels' tile order (gram_core.cuh: make_tiles and
// tile_coords, which every role of every CTA evaluates per tile).  For each
// shape, tile set and band width, t = 0 .. ntiles - 1 must give every tile of
// the set exactly once and nothing outside it:
//   kFull   every (row block, column block);
//   kUpper  column block tj holds row blocks 0 .. min(2 tj + 1, tr - 1);
//   kLower  row block ti holds column blocks 0 .. min(ti / 2, tc - 1).
// Built by nvcc and run on the host (no kernel is launched).  Prints "ok" and
// exits 0, or prints the first failure and exits 1.
#include "gram_core.cuh"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace gt;

static bool in_set(int mode, int64_t ti, int64_t tj, int64_t tr, int64_t tc) {
  if (mode == kFull) return true;
  if (mode == kUpper) return ti <= (2 * tj + 1 < tr - 1 ? 2 * tj + 1 : tr - 1);
  return tj <= (ti / 2 < tc - 1 ? ti / 2 : tc - 1);
}

static bool check(int64_t nr, int64_t nc, int mode, int64_t group) {
  const TileSpace ts = make_tiles(nr, nc, mode, group);
  std::vector<char> seen(size_t(ts.tr * ts.tc), 0);
  int64_t expect = 0;
  for (int64_t ti = 0; ti < ts.tr; ti++)
    for (int64_t tj = 0; tj < ts.tc; tj++) expect += in_set(mode, ti, tj, ts.tr, ts.tc);
  if (expect != ts.ntiles) {
    std::printf("FAIL nr=%lld nc=%lld mode=%d group=%lld: %lld tiles, %lld in the set\n",
                (long long)nr, (long long)nc, mode, (long long)group, (long long)ts.ntiles,
                (long long)expect);
    return false;
  }
  for (int64_t t = 0; t < ts.ntiles; t++) {
    int64_t ti = -1, tj = -1;
    tile_coords(ts, t, ti, tj);
    if (ti < 0 || ti >= ts.tr || tj < 0 || tj >= ts.tc || !in_set(mode, ti, tj, ts.tr, ts.tc) ||
        seen[size_t(ti * ts.tc + tj)]) {
      std::printf("FAIL nr=%lld nc=%lld mode=%d group=%lld: tile %lld -> (%lld, %lld)\n",
                  (long long)nr, (long long)nc, mode, (long long)group, (long long)t,
                  (long long)ti, (long long)tj);
      return false;
    }
    seen[size_t(ti * ts.tc + tj)] = 1;
  }
  return true;
}

int main() {
  const int64_t sizes[] = {1, 127, 128, 129, 255, 256, 257, 1000, 4095, 4096, 8192, 8193,
                           12000, 20000, 33000};
  const int64_t groups[] = {1, 2, 3, 4, 8, 12, 16};
  for (int64_t nr : sizes)
    for (int64_t g : groups) {
      // symmetric problems (nr == nc) in the upper and lower sets, and
      // two-set problems in the full set against a few column counts
      if (!check(nr, nr, kUpper, g) || !check(nr, nr, kLower, g)) return 1;
      for (int64_t nc : {int64_t(1), int64_t(300), int64_t(5000), nr + 77})
        if (!check(nr, nc, kFull, g)) return 1;
    }
  std::printf("ok\n");
  return 0;
}
