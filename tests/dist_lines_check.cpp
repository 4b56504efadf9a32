// Host check of the aligned-line tiling of the dist layout (dist_lines.cuh):
// for each n given, and output offsets 0, 7 and 31 floats within a line,
//   - pos and point are inverse, every point has one operand row;
//   - each tile's operand rows stay inside the permuted operand, its first
//     A row is >= -32, its columns ascend;
//   - every column of every tile starts each 32-row warp group on a line;
//   - the tiles enumerate each (row tile, super-block, class) once;
//   - with coverage (n <= 12000): every dist entry is computed exactly once.
// Prints "ok" and exits 0, or prints the first failure and exits 1.
#include "dist_lines.cuh"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace gt;

#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      std::printf("FAIL n=%lld o=%lld: ", (long long)n, (long long)o); \
      std::printf(__VA_ARGS__);          \
      std::printf("\n");                 \
      return false;                      \
    }                                    \
  } while (0)

static bool check(int64_t n, int64_t o) {
  DistLines dl;
  LineTiles lt;
  CHECK(make_dist_lines(n, uintptr_t(4096 + 4 * o), &dl), "make_dist_lines");
  CHECK(make_line_tiles(n, &lt), "make_line_tiles");
  const int64_t npb = lt.npb, Q = lt.nq, T = (n + 31) / 128 + 1;
  std::vector<int> owner(size_t(npb), -1);
  for (int64_t c = 0; c < n; c++) {
    const int64_t p = dl.pos(c);
    CHECK(p >= 0 && p < npb, "pos(%lld) = %lld", (long long)c, (long long)p);
    CHECK(dl.point(p) == c, "point(pos(%lld)) = %lld", (long long)c, (long long)dl.point(p));
    CHECK(owner[size_t(p)] < 0, "row %lld taken twice", (long long)p);
    owner[size_t(p)] = int(c);
  }
  for (int64_t p = 0; p < npb; p++)
    CHECK((owner[size_t(p)] >= 0) == (dl.point(p) < n), "padding row %lld", (long long)p);
  std::vector<uint8_t> seen(size_t(T * Q * 32), 0);
  const bool cover = n <= 12000;
  std::vector<uint8_t> hits(cover ? size_t(n * (n - 1) / 2) : 0, 0);
  for (uint32_t u = 0; u < lt.ntiles; u++) {
    int64_t row0, col0;
    lt.decode(u, row0, col0);
    const int64_t k = (col0 >> 8) & 31, q = col0 >> 13;
    const int64_t t = (row0 - k + 32) / 128;
    CHECK(row0 == k - 32 + 128 * t, "tile %u row0 %lld", u, (long long)row0);
    CHECK(t >= 0 && t < T && q >= 0 && q < Q, "tile %u (t %lld, q %lld)", u, (long long)t,
          (long long)q);
    CHECK(q <= t / 64 || t >= 64 * (Q - 1), "tile %u q beyond its row tile", u);
    CHECK(col0 % 256 == 0 && col0 + 256 <= npb, "tile %u col0 %lld", u, (long long)col0);
    uint8_t &s = seen[size_t((t * Q + q) * 32 + k)];
    CHECK(s == 0, "tile (t %lld, q %lld, k %lld) twice", (long long)t, (long long)q, (long long)k);
    s = 1;
    int64_t prev = -1;
    for (int64_t j = 0; j < 256; j++) {
      const int64_t c = dl.point(col0 + j);
      CHECK(c >= prev, "tile %u columns not ascending at %lld", u, (long long)j);
      prev = c;
      if (c >= n) continue;
      const int64_t base = n * c - c * (c + 1) / 2 - c - 1;
      for (int64_t w = 0; w < 4; w++)
        CHECK((((o + base + row0 + 32 * w) % 32) + 32) % 32 == 0,
              "tile %u column %lld warp %lld not on a line", u, (long long)c, (long long)w);
      if (!cover) continue;
      for (int64_t i = 0; i < 128; i++) {
        const int64_t r = row0 + i;
        if (c < r && r < n) hits[size_t(base + r)]++;
      }
    }
  }
  for (int64_t t = 0; t < T; t++)
    for (int64_t q = 0; q < Q; q++) {
      const bool want = q <= t / 64;
      for (int64_t k = 0; k < 32; k++)
        CHECK(bool(seen[size_t((t * Q + q) * 32 + k)]) == want, "tile (t %lld, q %lld, k %lld) %s",
              (long long)t, (long long)q, (long long)k, want ? "missing" : "extra");
    }
  for (size_t e = 0; e < hits.size(); e++) CHECK(hits[e] == 1, "entry %zu computed %d times", e, hits[e]);
  return true;
}

int main(int argc, char **argv) {
  for (int a = 1; a < argc; a++) {
    const int64_t n = std::atoll(argv[a]);
    for (int64_t o : {0, 7, 31})
      if (!check(n, o)) return 1;
  }
  std::printf("ok\n");
  return 0;
}
