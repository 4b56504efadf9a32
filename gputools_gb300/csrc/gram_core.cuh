// gram_core.cuh -- pieces shared by the tcgen05 Gram kernels (gram_tc.cu,
// gram_exact.cu): the tile space of one problem and its tile order, the
// epilogue context, the Pearson finish (r, t-score and pair count written in
// both orientations), and the work sources that tell every role of a
// persistent kernel which tile it handles next.
#pragma once

#include "common.cuh"
#include "kernels.cuh"
#include "tc_ptx.cuh"

#include <cuda.h>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <type_traits>
#include <vector>

namespace gt {

namespace {

constexpr int kBM = 128, kBN = 256;
constexpr uint64_t kDrainLimitNs = 200000000ull;  // 0.2 s for in-flight work at exit
constexpr int kKPad = 64;                         // K padding of the operand planes
constexpr int kMaxSmem = 232448;                  // dynamic shared memory per CTA (227 KB)
constexpr int kEpiTileFloats = 32 * 33;           // one warp's padded 32 x 32 staging tile

// The bounded-wait settings of a launch on the current device.
inline int make_wait_cfg(tc::WaitCfg *wc) {
  GT_TRY(device_error_word(&wc->err));
  wc->limit_ns = wait_limit_ns();
  wc->hint_ns = wait_sleep_hint_ns();
  return GT_OK;
}

// ----------------------------------------------------------------- tiling
// Tile sets.  kFull: every (row block, column block).  kUpper (symmetric
// problems whose entries r < c are wanted): column block tj holds row blocks
// 0 .. min(2 tj + 1, tr - 1), the 128-row blocks that reach the upper
// triangle of a 256-column block.  kLower (entries c < r): row block ti holds
// column blocks 0 .. min(ti / 2, tc - 1), enumerated row by row.
enum TileMode { kFull = 0, kUpper = 1, kLower = 2 };

struct TileSpace {
  int64_t tr, tc;    // row blocks (128), column blocks (256)
  int64_t j0;        // upper: column blocks whose tile count is 2*tj + 2
  int64_t ntiles;    // below 2^31
  int64_t group;     // upper / full: column blocks per band of the tile order (power of two)
  int group_log2;
  int symmetric;     // TileMode
};

// Tile order.  Column blocks are grouped into bands of `group` (a power of
// two); a band's tiles are consecutive, row block by row block, so the CTAs
// working at one time share a few operand panels in L2: the band's B panels
// stay resident while its A panels stream past once per band instead of once
// per column block.  Every role of every CTA evaluates this per tile, so it
// runs in 32-bit arithmetic (the host keeps tile counts below 2^31): 64-bit
// integer division is a long software sequence on the GPU.
__host__ __device__ inline void tile_coords(const TileSpace &ts, int64_t t64, int64_t &ti,
                                            int64_t &tj) {
  const uint32_t t = uint32_t(t64), tr = uint32_t(ts.tr), tc = uint32_t(ts.tc);
  const uint32_t G = uint32_t(ts.group), lg = uint32_t(ts.group_log2);
  if (ts.symmetric == kLower) {
    // row pairs (2m, 2m + 1) hold m + 1 tiles each while m + 1 <= tc; rows
    // from 2 tc on hold tc tiles
    const uint32_t head = tc * (tc + 1);
    if (t < head) {
      int32_t m = int32_t((sqrtf(float(t) * 4.f + 1.f) - 1.f) * 0.5f);
      if (m < 0) m = 0;
      while (uint32_t(m + 1) * uint32_t(m + 2) <= t) m++;
      while (uint32_t(m) * uint32_t(m + 1) > t) m--;
      const uint32_t u = t - uint32_t(m) * uint32_t(m + 1), w = uint32_t(m) + 1;
      const uint32_t e = u >= w ? 1u : 0u;
      ti = 2 * uint32_t(m) + e;
      tj = u - e * w;
    } else {
      const uint32_t u = t - head;
      const uint32_t i = u / tc;
      ti = 2 * tc + i;
      tj = u - i * tc;
    }
    return;
  }
  if (ts.symmetric == kFull) {
    const uint32_t c0 = (t / (tr << lg)) << lg;
    const uint32_t g = (tc - c0) < G ? (tc - c0) : G;
    const uint32_t u = t - c0 * tr;
    const uint32_t i = u / g;
    ti = i;
    tj = c0 + (u - i * g);
    return;
  }
  // column block of t in column-major order, hence its band
  const uint32_t j0 = uint32_t(ts.j0);
  const uint32_t head = j0 * (j0 + 1);
  uint32_t col;
  if (t < head) {
    // float estimate, corrected in integers
    int32_t j = int32_t((sqrtf(float(t) * 4.f + 1.f) - 1.f) * 0.5f);
    if (j < 0) j = 0;
    while (uint32_t(j + 1) * uint32_t(j + 2) <= t) j++;
    while (uint32_t(j) * uint32_t(j + 1) > t) j--;
    col = uint32_t(j);
  } else {
    col = j0 + (t - head) / tr;
  }
  const uint32_t c0 = (col >> lg) << lg;
  const uint32_t c1 = (c0 + G) < tc ? (c0 + G) : tc;
  const uint32_t g = c1 - c0;
  const uint32_t pre = c0 <= j0 ? c0 * (c0 + 1) : head + (c0 - j0) * tr;
  uint32_t u = t - pre;
  // rows 0 .. 2 c0 + 1 meet every column block of the band
  const uint32_t F = (2 * c0 + 2) < tr ? (2 * c0 + 2) : tr;
  if (u < F * g) {
    const uint32_t i = u / g;
    ti = i;
    tj = c0 + (u - i * g);
    return;
  }
  // row F + w meets the last g - 1 - floor(w / 2) column blocks
  u -= F * g;
  for (uint32_t w = 0;; w++) {
    const uint32_t cnt = g - 1 - w / 2;
    if (u < cnt) {
      ti = F + w;
      tj = c1 - cnt + u;
      return;
    }
    u -= cnt;
  }
}

inline TileSpace make_tiles(int64_t nr, int64_t nc, int mode, int64_t group) {
  TileSpace ts;
  ts.tr = cdiv(nr, kBM);
  ts.tc = cdiv(nc, kBN);
  ts.symmetric = mode;
  ts.group_log2 = 0;
  while ((int64_t(2) << ts.group_log2) <= group) ts.group_log2++;
  ts.group = int64_t(1) << ts.group_log2;
  if (mode == kLower) {
    ts.j0 = 0;
    ts.group = 1;
    ts.group_log2 = 0;
    if (ts.tr <= 2 * ts.tc) {
      const int64_t m = ts.tr / 2, e = ts.tr % 2;
      ts.ntiles = m * (m + 1) + e * (m + 1);
    } else {
      ts.ntiles = ts.tc * (ts.tc + 1) + (ts.tr - 2 * ts.tc) * ts.tc;
    }
  } else if (mode == kUpper) {
    ts.j0 = ts.tr / 2;
    if (ts.j0 > ts.tc) ts.j0 = ts.tc;
    ts.ntiles = ts.j0 * (ts.j0 + 1) + (ts.tc - ts.j0) * ts.tr;
  } else {
    ts.j0 = 0;
    ts.ntiles = ts.tr * ts.tc;
  }
  return ts;
}

// Band width for operand planes of `panel_bytes` per 256-row B panel: as
// many B panels as fit in about 48 MB of L2, at most 16 (make_tiles rounds
// it down to a power of two).  Measured at 20000 x 4096: the error-free Gram
// (6 MB panels) with groups of 1 / 2 / 4 / 8 / 16 panels 7.13 / 6.91 / 6.76 /
// 6.59 / 6.74 ms, the f16x3 Gram (4 MB panels) 3.45 ms with 8, 3.52 with 16.
inline int64_t band_group(int64_t panel_bytes) {
  const char *e = std::getenv("GT_TC_GROUP");
  if (e && std::atoi(e) > 0) return std::atoi(e);
  const int64_t g = (int64_t(48) << 20) / (panel_bytes > 0 ? panel_bytes : 1);
  return g < 1 ? 1 : (g > 16 ? 16 : g);
}

// ----------------------------------------------------------------- finishes
// Each finish handles a warp's 32 x 32 block: lane = row r (consecutive rows
// across lanes), g[j] = entry (r, c0 + j).  The epilogue context carries the
// warp's staging tile and the rows / columns of its part of the tile; after
// the last block of a tile the epilogue calls flush().

constexpr int kEuclidList = 64;  // pending near-zero pairs per epilogue warp

constexpr int kEuclidCols = 64;  // columns per epilogue warp of the Euclidean kernels

// Per-warp state of the epilogue.  Only what changes per tile lives here;
// the list and the column norms sit at fixed offsets after the staging tile.
struct EpiCtx {
  float *wsm;       // 32 x 33 staging tile, then (Euclidean) the list and column norms
  float2 me;        // this lane's row's {norm, scale} (Euclidean)
  int nlist;        // warp-uniform: entries in the shared-memory list
  int gcount;       // warp-uniform: entries in the warp's region of a global list
  int64_t rbase;    // first row of the warp's 32 rows
  int64_t col0;     // first column of the warp's columns
  // kEuclidList entries: (row - rbase) << 8 | (col - col0), or finish-defined
  __device__ __forceinline__ uint32_t *list() const {
    return reinterpret_cast<uint32_t *>(wsm + kEpiTileFloats);
  }
  // the warp's kEuclidCols columns' {norm, scale} (Euclidean)
  __device__ __forceinline__ float2 *cnrm() const {
    return reinterpret_cast<float2 *>(wsm + kEpiTileFloats + kEuclidList);
  }
};

// Whether a finish takes a block from the warp's staging tile (block()), not
// only from registers (operator()).
template <class Fin, class = void>
struct staged_block : std::false_type {};
template <class Fin>
struct staged_block<Fin, std::void_t<decltype(Fin::kStagedBlock)>>
    : std::integral_constant<bool, Fin::kStagedBlock> {};

__device__ __forceinline__ float clamp_r(float r) { return r > 1.f ? 1.f : (r < -1.f ? -1.f : r); }

// hostSignif's rule (src/correlation.cpp:51-64), t = r sqrt(n-2) / sqrt(1-r^2)
// with sqrt(n-2) precomputed and a hardware reciprocal square root.
__device__ __forceinline__ float signif_fast(float r, float sq_nm2) {
  if (r >= 0.999f) return 10000.0f;
  return r * sq_nm2 * tc::rsqrt_approx(1.f - r * r);
}

struct PearsonFinish {
  static constexpr bool kStagedBlock = true;  // has block(): entries from the staging tile
  float *corr, *ts, *pairs;
  int64_t ld, nr, nc;
  float npairs, sq_nm2;
  float gscale;  // removes the operand scales (2^-28 for f16x3, else 1)
  int symmetric;
  const int *gate = nullptr;  // when set, the kernel does nothing unless *gate == 0

  __device__ __forceinline__ bool skip() const { return gate && *gate != 0; }

  __device__ __forceinline__ void put(float *pc, float *pt, float *pp, float v) const {
    if (corr) tc::st_stream(pc, v);
    if (ts) tc::st_stream(pt, signif_fast(v, sq_nm2));
    if (pairs) tc::st_stream(pp, npairs);
  }

  // A block from registers: g[j] = entry (r, c0 + j), lanes on consecutive rows.
  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < 32; j++) ctx.wsm[lane * 33 + j] = g[j];
    __syncwarp();
    block(r, c0, ctx);
  }

  // Whether the block of rows rbase .. rbase + 31, columns c0 .. c0 + 31 has
  // anything to write: not past the problem's edge and (symmetric) not
  // entirely below the diagonal, whose entries the mirror stores of other
  // blocks write.
  __device__ __forceinline__ bool block_live(int64_t rbase, int64_t c0) const {
    return c0 < nc && rbase < nr && !(symmetric && rbase > c0 + 31);
  }

  // A block staged in the warp's tile: wsm[lane * 33 + j] = entry (r, c0 + j).
  // Both orientations read the tile (the padding keeps either read free of
  // bank conflicts), so the body is compact: loops of four, not unrolled
  // copies per entry.  Ends with the warp converged and the tile free.
  __device__ void block(int64_t r, int64_t c0, EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    const float *wsm = ctx.wsm;
    const int64_t rbase = r - lane;
    // interior block: every entry exists and (symmetric) lies above the diagonal
    const bool interior = (c0 + 31 < nc) && (symmetric ? (rbase + 31 < c0) : (rbase + 31 < nr));
    if (interior) {
      if (symmetric) {
        // mirror orientation: lanes hold consecutive rows of column c0 + j
        const int64_t o = c0 * ld + r;
        float *pc = corr + o, *pt = ts + o, *pp = pairs + o;
#pragma unroll 4
        for (int j = 0; j < 32; j++) {
          put(pc, pt, pp, clamp_r(wsm[lane * 33 + j] * gscale));
          pc += ld;
          pt += ld;
          pp += ld;
        }
      }
      const int64_t o = rbase * ld + c0 + lane;
      float *pc = corr + o, *pt = ts + o, *pp = pairs + o;
#pragma unroll 4
      for (int i = 0; i < 32; i++) {
        put(pc, pt, pp, clamp_r(wsm[i * 33 + lane] * gscale));
        pc += ld;
        pt += ld;
        pp += ld;
      }
      __syncwarp();
      return;
    }
    // Edge and diagonal blocks: the same loops with predicated stores.
    // Columns past nc (j >= jn) and rows past nr (i >= in_) are skipped; a
    // symmetric problem keeps entries on and above the diagonal.
    const int jn = nc - c0 >= 32 ? 32 : int(nc - c0);
    const int in_ = nr - rbase >= 32 ? 32 : int(nr - rbase);
    if (symmetric && r < nr) {
      int64_t o = c0 * ld + r;
      const int dj = int(r - c0);  // the lane's diagonal column, relative to c0
#pragma unroll 4
      for (int j = 0; j < 32; j++) {
        if (j < jn && j > dj) {
          const float v = clamp_r(wsm[lane * 33 + j] * gscale);
          if (corr) tc::st_stream(corr + o, v);
          if (ts) tc::st_stream(ts + o, signif_fast(v, sq_nm2));
          if (pairs) tc::st_stream(pairs + o, npairs);
        }
        o += ld;
      }
    }
    if (lane < jn) {
      const int64_t c = c0 + lane;
      const int64_t di = symmetric ? c - rbase : 31;  // rows i <= di are kept
      int64_t o = rbase * ld + c;
#pragma unroll 4
      for (int i = 0; i < 32; i++) {
        if (i < in_ && i <= di) {
          float v = clamp_r(wsm[i * 33 + lane] * gscale);
          if (symmetric && i == di && v == v) v = 1.f;
          if (corr) tc::st_stream(corr + o, v);
          if (ts) tc::st_stream(ts + o, signif_fast(v, sq_nm2));
          if (pairs) tc::st_stream(pairs + o, npairs);
        }
        o += ld;
      }
    }
    __syncwarp();
  }
  __device__ void begin_tile(int64_t, EpiCtx &) const {}
  __device__ void end_tile(EpiCtx &) const {}
  __device__ void drain(EpiCtx &) const {}
};

// ----------------------------------------------------------------- work sources
// A work source tells every role of the kernel, for the cursor-th tile of
// this CTA, which tensor maps to load from, the tile's row / column blocks,
// its number of k-blocks, and the finish to apply.
struct TileRef {
  const CUtensorMap *ma, *mb;
  int64_t row0, col0;  // first operand row of the A and B boxes (A may start below 0)
  int64_t nk, prob;
  int64_t k0 = 0;      // first k-block (a contraction whose K range is split)
};

// One problem: maps and finish as kernel parameters, tiles dealt round-robin.
template <class Fin>
struct SingleWork {
  CUtensorMap ma, mb;
  TileSpace ts;
  int64_t nk;
  Fin fin;
  __device__ bool tile(int64_t cursor, TileRef &ref) const {
    const int64_t t = int64_t(blockIdx.x) + cursor * int64_t(gridDim.x);
    if (t >= ts.ntiles) return false;
    int64_t ti, tj;
    tile_coords(ts, t, ti, tj);
    ref.row0 = ti * kBM;
    ref.col0 = tj * kBN;
    ref.ma = &ma;
    ref.mb = &mb;
    ref.nk = nk;
    ref.prob = 0;
    return true;
  }
  static constexpr bool kPrefetch = false;
  __device__ bool skip() const {
    if constexpr (std::is_same<Fin, PearsonFinish>::value) return fin.skip();
    return false;
  }
  __device__ const Fin &finish(const TileRef &) const { return fin; }
  __device__ void drain(EpiCtx &ctx) const { fin.drain(ctx); }
  __device__ void prefetch() const {
    tc::prefetch_tensormap(&ma);
    tc::prefetch_tensormap(&mb);
  }
};

// One problem whose tiles come from a table of (row0, col0) built on the host
// (a band of rows at a time, in the order the table lists them); the cursor
// looks each entry up a tile ahead.
template <class Fin>
struct TableWork {
  CUtensorMap ma, mb;
  const int2 *tiles;
  int64_t ntiles;
  int64_t nk;
  Fin fin;
  __device__ bool tile(int64_t cursor, TileRef &ref) const {
    const int64_t u = int64_t(blockIdx.x) + cursor * int64_t(gridDim.x);
    if (u >= ntiles) return false;
    const int2 t = tiles[u];
    ref.row0 = t.x;
    ref.col0 = t.y;
    ref.ma = &ma;
    ref.mb = &mb;
    ref.nk = nk;
    ref.prob = 0;
    return true;
  }
  static constexpr bool kPrefetch = true;
  __device__ bool skip() const {
    if constexpr (std::is_same<Fin, PearsonFinish>::value) return fin.skip();
    return false;
  }
  __device__ const Fin &finish(const TileRef &) const { return fin; }
  __device__ void drain(EpiCtx &ctx) const { fin.drain(ctx); }
  __device__ void prefetch() const {
    tc::prefetch_tensormap(&ma);
    tc::prefetch_tensormap(&mb);
  }
};

// The tiles (128 x 256) of a Pearson problem grouped in bands of row blocks:
// band b holds the tiles whose row block lies in [b * band_blocks,
// (b + 1) * band_blocks); for a symmetric problem only those meeting the
// upper triangle (row block ti <= 2 tj + 1).  Within a band, column block by
// column block.  After the bands 0 .. b have run, every row of band b is
// complete, mirror entries included (an entry (r, c), r <= c, is written by
// the tile of row r's block).  offsets[b] .. offsets[b + 1] index band b.
inline void band_tiles(int64_t nr, int64_t nc, bool symmetric, int64_t band_blocks,
                       std::vector<int2> &tiles, std::vector<int64_t> &offsets) {
  const int64_t tr = cdiv(nr, kBM), tc_ = cdiv(nc, kBN);
  tiles.clear();
  offsets.assign(1, 0);
  for (int64_t b0 = 0; b0 < tr; b0 += band_blocks) {
    const int64_t b1 = b0 + band_blocks < tr ? b0 + band_blocks : tr;
    for (int64_t tj = 0; tj < tc_; tj++)
      for (int64_t ti = b0; ti < b1; ti++)
        if (!symmetric || ti <= 2 * tj + 1)
          tiles.push_back(make_int2(int(ti * kBM), int(tj * kBN)));
    offsets.push_back(int64_t(tiles.size()));
  }
}

__device__ __forceinline__ int64_t find_segment(const int64_t *__restrict__ prefix, int64_t n,
                                                int64_t x) {
  int64_t lo = 0, hi = n;  // prefix has n + 1 entries; largest i with prefix[i] <= x
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (prefix[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// A batch of cor(x) problems: per-problem maps and finishes in device
// memory; each CTA walks its own host-balanced list of global tile ids.
struct PearsonBatchProblem {  // aligned as CUtensorMap
  CUtensorMap map_a, map_b;  // 128-row and 256-row boxes over the same planes
  TileSpace ts;
  int64_t nk;
  PearsonFinish fin;
};

// Each CTA walks its own list of tiles, built on the host: per tile one
// entry {problem, row0, col0, k-blocks}, so a lookup is one 16-byte load that
// the cursor issues a tile ahead.
struct PearsonBatchWork {
  static constexpr bool kWideEpi = true;  // sixteen epilogue warps with 32-wide K blocks
  const PearsonBatchProblem *probs;
  const int4 *table;     // the CTAs' tile lists, one after the other
  const int64_t *cta_off;  // CTA c's tiles: table[cta_off[c] .. cta_off[c + 1])
  __device__ bool tile(int64_t cursor, TileRef &ref) const {
    const int64_t idx = cta_off[blockIdx.x] + cursor;
    if (idx >= cta_off[blockIdx.x + 1]) return false;
    const int4 t = table[idx];
    const PearsonBatchProblem &pr = probs[t.x];
    ref.row0 = t.y;
    ref.col0 = t.z;
    ref.ma = &pr.map_a;
    ref.mb = &pr.map_b;
    ref.nk = t.w;
    ref.prob = t.x;
    return true;
  }
  // the next tile is looked up when reached: holding it costs the sixteen-warp
  // kernel (96 registers) spills that outweigh the lookup
  static constexpr bool kPrefetch = false;
  __device__ bool skip() const { return false; }
  __device__ PearsonFinish finish(const TileRef &ref) const { return probs[ref.prob].fin; }
  __device__ void drain(EpiCtx &) const {}
  __device__ void prefetch() const {}
};

// Walks this CTA's tiles first, first + step, ... of a work source.  With
// Work::kPrefetch it looks up the next tile while the current one is
// processed (the lookup is a global load); else it looks each tile up when it
// is reached, holding no second TileRef.
template <class Work, bool PREFETCH = Work::kPrefetch>
struct TileCursor {
  const Work &work;
  TileRef nref;
  int64_t cur;
  int step;
  bool have;
  __device__ TileCursor(const Work &w, int first, int stp) : work(w), cur(first), step(stp) {
    have = work.tile(cur, nref);
  }
  __device__ bool next(TileRef &ref) {
    if (!have) return false;
    ref = nref;
    cur += step;
    have = work.tile(cur, nref);
    return true;
  }
};
template <class Work>
struct TileCursor<Work, false> {
  const Work &work;
  int64_t cur;
  int step;
  __device__ TileCursor(const Work &w, int first, int stp) : work(w), cur(first), step(stp) {}
  __device__ bool next(TileRef &ref) {
    const bool got = work.tile(cur, ref);
    cur += step;
    return got;
  }
};

}  // namespace

}  // namespace gt
