// dist_lines.cuh -- the aligned-line tiling of R's dist layout used by the
// tensor-core Euclidean kernel; plain C++ on the host (the tiling test builds
// it with g++) and device code under nvcc.
//
// R's dist vector (what as.dist makes of the reference's full matrix,
// R/gpuHclust.R:29), the strict lower triangle by columns, holds entry
// (c, r), c < r, at base(c) + r with base(c) = n c - c (c + 1) / 2 - c - 1.
// A warp storing column c for 32 consecutive rows
// writes one whole 128-byte line exactly when the first row is congruent to
// cls(c) = -(o + base(c)) mod 32, o the output's offset in floats within its
// line; otherwise the store touches two lines, and the L2's write-request
// rate, not HBM, bounds the kernel.  base(c + 64) - base(c) =
// 64 (n - c - 1) - 2080 is a multiple of 32, so cls depends on c mod 64 only,
// and (triangular numbers being a complete residue system modulo 32) every
// class holds exactly two of any 64 consecutive columns; make_dist_lines
// checks both.
//
// The column operand is therefore permuted: super-block q (columns 8192 q ..
// 8192 q + 8191) becomes 32 runs of 256 operand rows, one per class, each in
// column order; the runs of the last super-block are padded.  Tile (t, q, k)
// pairs class k of super-block q with rows k - 32 + 128 t .. + 127, so each
// warp's 32 rows start on a line of every column of the tile.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GT_HD __host__ __device__ __forceinline__
#else
#define GT_HD inline
#endif

namespace gt {

constexpr int64_t kLineSuper = 8192;  // columns per super-block: 32 classes x 256

struct DistLines {
  uint8_t cls_rank[64];  // u = c mod 64: class << 1 | rank of u within its class
  uint8_t member[64];    // member[2 k + e]: the e-th u (ascending) of class k
  int64_t n;
  // operand row of column c
  GT_HD int64_t pos(int64_t c) const {
    const uint32_t cr = cls_rank[c & 63];
    return ((((c >> 13) << 5) + int64_t(cr >> 1)) << 8) + (((c & 8191) >> 6) << 1) + (cr & 1u);
  }
  // the same in 32-bit arithmetic (p and n below 2^31)
  GT_HD int32_t point32(uint32_t p) const {
    const uint32_t k = (p >> 8) & 31u, e = p & 255u;
    const int32_t c = int32_t(((p >> 13) << 13) + ((e >> 1) << 6) + member[2 * k + (e & 1u)]);
    return c < int32_t(n) ? c : int32_t(n);
  }
  // column of operand row p; n for padding rows
  GT_HD int64_t point(int64_t p) const {
    const int64_t k = (p >> 8) & 31, e = p & 255;
    const int64_t c = ((p >> 13) << 13) + ((e >> 1) << 6) + member[2 * k + (e & 1)];
    return c < n ? c : n;
  }
};

// Class tables for n points written at the float address `out`.  Returns
// false when the output is not float aligned or a class does not hold
// exactly two residues.
inline bool make_dist_lines(int64_t n, uintptr_t out, DistLines *dl) {
  if (out & 3u) return false;
  const int64_t o = int64_t((out >> 2) & 31u);
  int cnt[32] = {0};
  for (int64_t u = 0; u < 64; u++) {
    const int64_t base = n * u - u * (u + 1) / 2 - u - 1;
    const int64_t k = (((-(o + base)) % 32) + 32) % 32;
    if (cnt[k] >= 2) return false;
    dl->member[2 * k + cnt[k]] = uint8_t(u);
    dl->cls_rank[u] = uint8_t((k << 1) | cnt[k]);
    cnt[k]++;
  }
  dl->n = n;
  return true;
}

// Tile order: k fastest, then the super-blocks q <= t / 64 that reach row
// tile t, then t.  Row tiles 64 b .. 64 b + 63 hold b + 1 super-blocks each
// (while b + 1 <= Q), so 32 b (b + 1) (t, q) pairs precede row tile 64 b;
// from row tile 64 (Q - 1) on every row tile holds Q.  Row tiles run while
// k - 32 + 128 t <= n - 1 for k = 0.  Tiles whose rows all lie at or above
// their columns, or at or beyond n, are masked by the finish.  Decoding runs
// in 32-bit arithmetic (64-bit division is a long sequence on the GPU).
struct LineTiles {
  uint32_t nq;      // super-blocks Q
  uint32_t head;    // (t, q) pairs before row tile 64 (Q - 1): 32 (Q - 1) Q
  uint32_t ntiles;  // 32 x (t, q) pairs
  int64_t npb;      // operand rows of the permuted column operand: 8192 Q

  // first A row (may be negative, down to -32) and first B row of tile u
  GT_HD void decode(uint32_t u, int64_t &row0, int64_t &col0) const {
    const uint32_t k = u & 31u, v = u >> 5;
    uint32_t t, q;
    if (v < head) {
      int32_t b = int32_t((sqrtf(1.f + float(v) * 0.125f) - 1.f) * 0.5f);
      if (b < 0) b = 0;
      while (32u * uint32_t(b + 1) * uint32_t(b + 2) <= v) b++;
      while (32u * uint32_t(b) * uint32_t(b + 1) > v) b--;
      const uint32_t w = v - 32u * uint32_t(b) * uint32_t(b + 1), g = uint32_t(b) + 1u;
      const uint32_t i = w / g;
      t = 64u * uint32_t(b) + i;
      q = w - i * g;
    } else {
      const uint32_t w = v - head;
      const uint32_t i = w / nq;
      t = 64u * (nq - 1u) + i;
      q = w - i * nq;
    }
    row0 = int64_t(k) - 32 + 128 * int64_t(t);
    col0 = int64_t((q << 5) | k) << 8;
  }
};

// Tile counts for n >= 2 points; false when the tiles exceed 2^31 - 1.
inline bool make_line_tiles(int64_t n, LineTiles *lt) {
  const int64_t Q = (n + kLineSuper - 1) / kLineSuper;
  const int64_t T = (n + 31) / 128 + 1;
  if (n < 2 || T < 64 * (Q - 1)) return false;
  const int64_t pairs = 32 * (Q - 1) * Q + (T - 64 * (Q - 1)) * Q;
  if (32 * pairs > 2147483647LL) return false;
  lt->nq = uint32_t(Q);
  lt->head = uint32_t(32 * (Q - 1) * Q);
  lt->ntiles = uint32_t(32 * pairs);
  lt->npb = Q * kLineSuper;
  return true;
}

}  // namespace gt
