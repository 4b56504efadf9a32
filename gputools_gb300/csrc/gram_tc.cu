// gram_tc.cu -- split-bf16 Gram contractions on tcgen05 tensor cores, for
// Pearson (gpuCor "everything"), Euclidean distances (gpuDist) and the
// Pearson adjoint's GEMM.
//
// Reference: the contraction the reference performs as one n-length dot
// product per 16-thread block (inst/cuda/correlation.cu:248-292
// gpuPMCCNoTest) and as one (a-b)^2 loop per 32-thread block
// (inst/cuda/distance.cu:40-78).
//
// Operands.  Each value v (Pearson: the normalised column entry
// z = (x - mean)/||x - mean||; Euclidean: the centred coordinate) is split
// into 16-bit parts, each the round-to-nearest of the remainder of the
// previous ones.  The parts live in separate planes [part][row][k] (K
// contiguous, padded to a multiple of 64 with zeros).  The Gram entry is the
// sum of the part products of total order at most NSPLIT-1:
//   bf16x3: two bf16 parts, v0w0 + v0w1 + v1w0            (~2^-16 relative)
//   bf16x6: three bf16 parts, + v0w2 + v1w1 + v2w0        (float32-level)
//   f16x3:  two fp16 parts of v scaled by a power of two (Pearson: 2^14 for
//           every row, since |z| <= 1; Euclidean: per point, its largest
//           magnitude into [2^14, 2^15)), three products     (~2^-21)
// f16x3 costs what bf16x3 costs on the tensor core; the epilogue removes the
// scales exactly.
//
// Accumulation.  The tensor core's FP32 accumulation rounds every add toward
// zero, so its error grows linearly with the number of adds into one
// accumulator (measured: about 2^-25 |acc| per add).  When CHUNKED, K is
// split into chunks of `ckb` k-blocks; each chunk starts from zero in TMEM and
// the epilogue adds it into FP32 registers with round-to-nearest.
//
// Kernel.  Persistent, one CTA per SM, 10 warps:
//   warp 0      TMA producer: 3-D tensor loads (part plane, row block, K) of
//               the A (128-row) and B (256-row) tiles into a smem ring
//               (128- or 64-byte swizzle), completion tracked by mbarriers;
//   warp 1      allocates 512 TMEM columns (two 128 x 256 FP32 accumulators)
//               and one thread issues tcgen05.mma (M = 128, N = 256, K = 16)
//               for every part product, committing each smem stage back to
//               the producer and each finished chunk to the epilogue;
//   warps 2..9  epilogue: two warps per TMEM lane quarter, 128 columns each;
//               tcgen05.ld, then the fused Pearson / Euclidean / store finish,
//               while the MMAs fill the other accumulator.
// Symmetric problems (cor(x), gpuDist) schedule only the 128 x 256 tiles
// that meet the upper triangle and store each entry and its mirror.  Each
// warp writes rows through a padded 32 x 33 shared tile, so both orientations
// are stored with coalesced 128-byte transactions.
// Every mbarrier wait is bounded: on timeout the CTA raises an error word,
// drains its in-flight copies and MMAs, releases its TMEM and exits.
#include "common.cuh"
#include "dist_lines.cuh"
#include "gram_core.cuh"
#include "kernels.cuh"
#include "tc_ptx.cuh"
#include "stats.cuh"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <queue>
#include <type_traits>
#include <vector>

namespace gt {

namespace {

// Operands are the points centred by their column means (distances do not
// change).  The kernel runs the lower tile set: TMEM lane = point a, column =
// point b < a, so for a fixed column the 32 lanes of a warp hold consecutive
// points a, which are consecutive entries of one row of R's dist layout (and
// of one row of the full matrix's mirror orientation): those stores go out
// coalesced straight from registers.
// d^2 = |a|^2 + |b|^2 - 2 G with float norms (compensated sums); an entry
// whose d^2 is below tau * (|a|^2 + |b|^2), where rounding of the contraction
// could dominate, is recomputed from the original float points: the warp
// queues such pairs and recomputes four at a time, eight lanes per pair
// (float differences, squares with their FMA residuals, compensated
// float-pair sums), overwriting the estimate it stored first.  Exact
// duplicates come out exactly 0.
// Near-zero pairs of the Euclidean finishes.  A block's pending bits (bit
// 31 - k: entry (lane's row, column k of the block) is recomputed) go to the
// warp's list through fin.push(ctx, slot, lane, column offset in the warp's
// columns); a full list is flushed at once.
template <class Fin>
__device__ __forceinline__ void euclid_queue(const Fin &fin, unsigned pend, uint32_t cofs,
                                             EpiCtx &ctx) {
  const unsigned FULLM = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  while (__any_sync(FULLM, pend != 0u)) {
    const int cnt = __popc(pend);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULLM, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(FULLM, incl, 31);
    const int room = kEuclidList - ctx.nlist;
    const int start = incl - cnt;
    int take = room - start;
    take = take < 0 ? 0 : (take > cnt ? cnt : take);
    for (int t = 0; t < take; t++) {
      const int bit = __ffs(int(pend)) - 1;
      pend &= pend - 1u;
      fin.push(ctx, ctx.nlist + start + t, lane, cofs + uint32_t(31 - bit));
    }
    ctx.nlist += total < room ? total : room;
    if (ctx.nlist == kEuclidList) fin.flush(ctx);
  }
}

__device__ __forceinline__ void sq_add(float d, FloatPairSum &acc, float &res) {
  const float q = d * d;
  res += fmaf(d, d, -q);
  acc.add(q);
}

// |a_i - a_j|^2 from the float points, compensated: each of the 8 lanes of
// a group (sub = lane & 7) sums every 8th coordinate difference squared, the
// group combines the partial pairs; every lane of the group gets the sum.
__device__ __forceinline__ float pair_sq_dist(const float *__restrict__ pts, int64_t dim, int vec4,
                                              int64_t i, int64_t j, int sub) {
  const unsigned FULLM = 0xffffffffu;
  const float *pa = pts + i * dim, *pb = pts + j * dim;
  FloatPairSum acc;
  float res = 0.f;
  if (vec4) {
    const float4 *a4 = reinterpret_cast<const float4 *>(pa);
    const float4 *b4 = reinterpret_cast<const float4 *>(pb);
    const int64_t d4 = dim >> 2;
#pragma unroll 4
    for (int64_t k = sub; k < d4; k += 8) {
      const float4 x = a4[k], y = b4[k];
      sq_add(x.x - y.x, acc, res);
      sq_add(x.y - y.y, acc, res);
      sq_add(x.z - y.z, acc, res);
      sq_add(x.w - y.w, acc, res);
    }
  } else {
    for (int64_t k = sub; k < dim; k += 8) sq_add(pa[k] - pb[k], acc, res);
  }
  float hi = acc.hi, lo = acc.lo + res;
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(FULLM, hi, o), ol = __shfl_xor_sync(FULLM, lo, o);
    const float t = hi + oh, bp = t - hi;
    lo = (lo + ol) + ((hi - (t - bp)) + (oh - bp));
    hi = t;
  }
  return hi + lo;
}

// Recomputes the queued pairs: a group of 8 lanes per pair, 4 pairs per
// round.  fin.entry(ctx, slot, i, j) reads a list entry as its pair of points.
template <class Fin>
__device__ void euclid_flush(const Fin &fin, EpiCtx &ctx) {
  const int lane = threadIdx.x & 31, grp = lane >> 3, sub = lane & 7;
  __syncwarp();
  for (int b = 0; b < ctx.nlist; b += 4) {
    const int idx = b + grp;
    const bool act = idx < ctx.nlist;
    int64_t i, j;
    fin.entry(ctx, act ? idx : b, i, j);
    const float d2 = pair_sq_dist(fin.pts, fin.dim, fin.vec4, i, j, sub);
    if (act && sub == 0) fin.store_pair(i, j, sqrtf(d2));
  }
  ctx.nlist = 0;
  __syncwarp();
}

struct EuclidFinish {
  const float2 *nrm;  // per point {|c|^2, 2^-s} (s its f16x3 scale exponent, else 0),
                      // zero padded to a multiple of 256 points
  const float *pts;
  float *out;
  int64_t n, dim;
  int layout;  // GT_LAYOUT_FULL / GT_LAYOUT_DIST
  float tau;
  int vec4;    // pts 16-byte aligned and dim % 4 == 0

  __device__ __forceinline__ int64_t dist_index(int64_t i, int64_t j) const {  // i < j
    return n * i - i * (i + 1) / 2 - i - 1 + j;
  }

  // The lane's point values and the warp's column values for this tile.
  __device__ void begin_tile(int64_t r, EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    ctx.me = nrm[r];
    for (int k = lane; k < kEuclidCols; k += 32) ctx.cnrm()[k] = nrm[ctx.col0 + k];
    __syncwarp();
  }

  // Block of points a = r (lanes) against b = c0 + k (k = 0..31), b < a.
  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    float *wsm = ctx.wsm;
    const int64_t rbase = r - lane;
    const float na = ctx.me.x, ra = -2.f * ctx.me.y;
    // the block's column values (shared-memory broadcasts)
    const float2 *cv = ctx.cnrm() + (c0 - ctx.col0);
    const bool full = layout == GT_LAYOUT_FULL;
    // interior block: every column below every row, every row < n
    const bool interior = (c0 + 31 < rbase) && (rbase + 31 < n);
    unsigned pend = 0u;  // bit 31 - k: entry (r, c0 + k) is recomputed
    if (interior) {
      // row c0 + k of the dist layout (or of the full matrix), column r
      float *o = out + (full ? c0 * n + r : dist_index(c0, r));
      const int64_t step0 = full ? n : n - c0 - 2;
#pragma unroll
      for (int k = 0; k < 32; k++) {
        const float2 cj = cv[k];
        const float s = na + cj.x;
        const float d2 = fmaf(ra * cj.y, g[k], s);
        // (pend << 1) | sign of d2 - tau s, in one funnel shift
        pend = __funnelshift_l(__float_as_uint(fmaf(-tau, s, d2)), pend, 1);
        const float v = tc::sqrt_approx(fabsf(d2));
        *o = v;
        o += full ? step0 : step0 - k;
        if (full) wsm[lane * 33 + k] = v;
      }
      if (full) {
        // row orientation (r, c0 + k) through the staging tile
        __syncwarp();
        float *q = out + (rbase * n + c0 + lane);
#pragma unroll 8
        for (int i = 0; i < 32; i++) {
          *q = wsm[i * 33 + lane];
          q += n;
        }
      }
    } else {
      // this lane's row uses columns c0 + k < r, r < n
      const int64_t hi64 = r - c0;
      const int khi = r >= n ? 0 : (hi64 > 32 ? 32 : (hi64 < 0 ? 0 : int(hi64)));
#pragma unroll
      for (int k = 0; k < 32; k++) {
        const float2 cj = cv[k];
        const float s = na + cj.x;
        const float d2 = fmaf(ra * cj.y, g[k], s);
        const bool valid = k < khi;
        pend = (pend << 1) | unsigned(valid & (d2 < tau * s));
        const float v = valid ? tc::sqrt_approx(fabsf(d2)) : 0.f;
        wsm[lane * 33 + k] = v;
        if (valid) out[full ? (c0 + k) * n + r : dist_index(c0 + k, r)] = v;
      }
      if (full) {
        __syncwarp();
        const int64_t c = c0 + lane;
        for (int i = 0; i < 32; i++) {
          const int64_t ri = rbase + i;
          if (ri >= n) break;
          if (c < ri) out[ri * n + c] = wsm[i * 33 + lane];
          else if (c == ri) out[ri * n + c] = 0.f;
        }
      }
    }
    __syncwarp();
    // queue the pairs to recompute (after their estimates are stored)
    euclid_queue(*this, pend, uint32_t(c0 - ctx.col0), ctx);
  }

  // list entry: lane << 8 | column offset, relative to the current tile
  __device__ __forceinline__ void push(EpiCtx &ctx, int slot, int lane, uint32_t ofs) const {
    ctx.list()[slot] = (uint32_t(lane) << 8) | ofs;
  }
  __device__ __forceinline__ void entry(const EpiCtx &ctx, int slot, int64_t &i, int64_t &j) const {
    const uint32_t e = ctx.list()[slot];
    i = ctx.rbase + int64_t(e >> 8);
    j = ctx.col0 + int64_t(e & 255u);
  }
  __device__ __forceinline__ void store_pair(int64_t i, int64_t j, float d) const {
    if (layout == GT_LAYOUT_FULL) {
      out[i * n + j] = d;
      out[j * n + i] = d;
    } else {
      out[i < j ? dist_index(i, j) : dist_index(j, i)] = d;
    }
  }
  __device__ void flush(EpiCtx &ctx) const { euclid_flush(*this, ctx); }
  __device__ void end_tile(EpiCtx &ctx) const { flush(ctx); }
  __device__ void drain(EpiCtx &) const {}
};

// ----------------------------------------------------------------- aligned dist lines
// The dist layout through aligned lines.  The warp's columns sit in its
// staging tile, which this finish does not otherwise use: point ids, and the
// offsets base(c) - base(c_first) of their dist columns from the warp's first
// column (64 columns of one class span at most 4096 points, so the offsets
// fit 32 bits), and the base of that first column, all copied from the
// tables the split kernel writes.  The pending pairs follow them in the
// staging tile.
struct EuclidLineFinish {
  static constexpr int kCols = kEuclidCols;  // columns per epilogue warp
  const float2 *nrm;  // per point {|c|^2, 2^-s}
  const int4 *colinfo;       // per operand column: point, base offset in its group, norm, scale
  const int64_t *groupbase;  // per kCols operand columns: base of the group's first point
  const float *pts;
  float *out;
  int64_t n, dim;
  float tau;
  int vec4;
  int2 *pair_list;    // [CTA][epilogue warp][pair_cap] pending pairs (row, column)
  int *pair_count;    // [CTA][epilogue warp] pairs listed, written at the end
  int pair_cap, epi;

  // the warp's staging tile: point ids, offsets, pending pairs, the first
  // column's base, the columns' {norm, scale}
  __device__ __forceinline__ static int *col_ids(const EpiCtx &ctx) {
    return reinterpret_cast<int *>(ctx.wsm);
  }
  __device__ __forceinline__ static int *col_offs(const EpiCtx &ctx) {
    return reinterpret_cast<int *>(ctx.wsm) + kCols;
  }
  __device__ __forceinline__ static int2 *pairs(const EpiCtx &ctx) {
    return reinterpret_cast<int2 *>(ctx.wsm + 2 * kCols);  // kEuclidList entries
  }
  __device__ __forceinline__ static int64_t *first_base(const EpiCtx &ctx) {
    return reinterpret_cast<int64_t *>(ctx.wsm + 2 * kCols + 2 * kEuclidList);
  }
  __device__ __forceinline__ static float2 *col_nrm(const EpiCtx &ctx) {
    return reinterpret_cast<float2 *>(ctx.wsm + 2 * kCols + 2 * kEuclidList + 8);
  }
  static_assert(2 * kCols + 2 * kEuclidList + 8 + 2 * kCols <= kEpiTileFloats,
                "the columns fit the staging tile");
  // this warp's region of the global pair list (epilogue warps follow the
  // producer and MMA warps)
  __device__ __forceinline__ int64_t region_index() const {
    return int64_t(blockIdx.x) * epi + (int(threadIdx.x >> 5) - 2);
  }
  __device__ __forceinline__ int2 *region() const { return pair_list + region_index() * pair_cap; }
  __device__ __forceinline__ int64_t base(int64_t c) const { return n * c - c * (c + 1) / 2 - c - 1; }

  __device__ void begin_tile(int64_t r, EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    ctx.me = (r >= 0 && r < n) ? nrm[r] : make_float2(0.f, 0.f);
    if (lane == 0) *first_base(ctx) = groupbase[ctx.col0 / kCols];
    int *cid = col_ids(ctx);
    int *cof = col_offs(ctx);
    float2 *cn = col_nrm(ctx);
#pragma unroll
    for (int k = lane; k < kCols; k += 32) {
      const int4 ci = colinfo[ctx.col0 + k];
      cid[k] = ci.x;
      cof[k] = ci.y;
      cn[k] = make_float2(__int_as_float(ci.z), __int_as_float(ci.w));
    }
    __syncwarp();
  }

  // Rows r (lanes) against the block's 32 columns (ascending points).
  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    const int off = int(c0 - ctx.col0);
    const int *cid = col_ids(ctx) + off;
    const int4 *cof4 = reinterpret_cast<const int4 *>(col_offs(ctx) + off);
    const float4 *cv4 = reinterpret_cast<const float4 *>(col_nrm(ctx) + off);
    const int64_t rbase = r - lane;
    const float na = ctx.me.x, ra = -2.f * ctx.me.y;
    float *const orow = out + (*first_base(ctx) + r);
    // interior block: every column below every row, every row < n
    const bool interior = (int64_t(cid[31]) < rbase) && (rbase + 31 < n);
    unsigned pend = 0u;
    if (interior) {
#pragma unroll
      for (int k4 = 0; k4 < 8; k4++) {
        const int4 o4 = cof4[k4];
        const float4 ca = cv4[2 * k4], cb = cv4[2 * k4 + 1];
        const float cn[4] = {ca.x, ca.z, cb.x, cb.z}, cs[4] = {ca.y, ca.w, cb.y, cb.w};
        const int co[4] = {o4.x, o4.y, o4.z, o4.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const float s = na + cn[e];
          const float d2 = fmaf(ra * cs[e], g[4 * k4 + e], s);
          // (pend << 1) | sign of d2 - tau s, in one funnel shift
          pend = __funnelshift_l(__float_as_uint(fmaf(-tau, s, d2)), pend, 1);
          tc::st_stream(orow + co[e], tc::sqrt_approx(fabsf(d2)));
        }
      }
    } else {
#pragma unroll
      for (int k4 = 0; k4 < 8; k4++) {
        const int4 o4 = cof4[k4];
        const float4 ca = cv4[2 * k4], cb = cv4[2 * k4 + 1];
        const float cn[4] = {ca.x, ca.z, cb.x, cb.z}, cs[4] = {ca.y, ca.w, cb.y, cb.w};
        const int co[4] = {o4.x, o4.y, o4.z, o4.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const float s = na + cn[e];
          const float d2 = fmaf(ra * cs[e], g[4 * k4 + e], s);
          const bool valid = (int64_t(cid[4 * k4 + e]) < r) && (r < n);
          pend = (pend << 1) | unsigned(valid & (d2 < tau * s));
          if (valid) tc::st_stream(orow + co[e], tc::sqrt_approx(fabsf(d2)));
        }
      }
    }
    __syncwarp();
    queue(pend, off, ctx);
  }

  // Pending pairs go to the warp's region of the global list (recomputed by
  // euclid_fixup_kernel after this kernel); once the region is full, to the
  // shared-memory list that the warp recomputes itself.
  __device__ __forceinline__ void queue(unsigned pend, int off, EpiCtx &ctx) const {
    const unsigned FULLM = 0xffffffffu;
    const unsigned lanes = __ballot_sync(FULLM, pend != 0u);
    if (!lanes) return;
    const int lane = threadIdx.x & 31;
    // usual case: at most one pending entry per lane; slots by lane rank
    if (!__any_sync(FULLM, (pend & (pend - 1u)) != 0u)) {
      const int total = __popc(lanes);
      if (ctx.gcount + total <= pair_cap) {
        if (pend) {
          const int slot = ctx.gcount + __popc(lanes & ((1u << lane) - 1u));
          region()[slot] =
              make_int2(int(ctx.rbase) + lane, col_ids(ctx)[off + 31 - (__ffs(int(pend)) - 1)]);
        }
        ctx.gcount += total;
        return;
      }
    }
    const int cnt = __popc(pend);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULLM, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(FULLM, incl, 31);
    if (ctx.gcount + total <= pair_cap) {
      int2 *dst = region() + (ctx.gcount + incl - cnt);
      const int row = int(ctx.rbase) + lane;
      const int *cid = col_ids(ctx) + off;
      while (pend) {
        const int bit = __ffs(int(pend)) - 1;
        pend &= pend - 1u;
        *dst++ = make_int2(row, cid[31 - bit]);
      }
      ctx.gcount += total;
      return;
    }
    euclid_queue(*this, pend, uint32_t(off), ctx);
  }

  // list entry: the absolute pair (row, column), so that pairs wait across
  // tiles and a warp recomputes only full lists (and its rest at the end)
  __device__ __forceinline__ void push(EpiCtx &ctx, int slot, int lane, uint32_t ofs) const {
    pairs(ctx)[slot] = make_int2(int(ctx.rbase) + lane, col_ids(ctx)[ofs]);
  }
  __device__ __forceinline__ void entry(const EpiCtx &ctx, int slot, int64_t &i, int64_t &j) const {
    const int2 e = pairs(ctx)[slot];
    i = e.x;
    j = e.y;
  }
  __device__ __forceinline__ void store_pair(int64_t i, int64_t j, float d) const {
    out[base(j) + i] = d;  // i is the row (the larger point), j the column
  }
  __device__ void flush(EpiCtx &ctx) const { euclid_flush(*this, ctx); }
  __device__ void end_tile(EpiCtx &) const {}
  __device__ void drain(EpiCtx &ctx) const {
    if ((threadIdx.x & 31) == 0) pair_count[region_index()] = ctx.gcount;
    if (ctx.nlist) flush(ctx);
  }
};

// B-spline mutual information (inst/cuda/mi.cu:115-152 get_mi): rows and
// columns are (variable, bin) with 2^lg bins per variable (zero padded), the
// Gram entry times gscale / nsamples is the joint probability p_ab of the
// two variables' bins.  A 32 x 32 block holds whole bin blocks: each lane sums
// p log2 p over a column variable's bins, the lanes of one row variable add
// their sums, and MI = that sum + H(x) + H(y) goes to out[y * ldo + x] (the
// reference layout; with symmetric, pairs x <= y and their mirror).
template <int LG>  // log2 of the bins per variable: a compact body per bin count
struct MiFinish {
  float *out;
  const float *hx, *hy;  // entropies of the row and column variables
  int64_t nx, ny, ldo;   // variables, row length of out
  float pscale;          // gscale / nsamples
  int symmetric;
  unsigned colmask;      // bit j: column j of a 32-column block is a real bin (not padding)
  static constexpr int kNb = 1 << LG;

  __device__ __forceinline__ static float plog2p(float p) { return p > 0.f ? p * __log2f(p) : 0.f; }

  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], EpiCtx &) const {
    const int lane = threadIdx.x & 31;
    const int64_t x = r >> LG;
    float t[32];
    // padding bins are zero columns: skipped (the same positions in every lane)
#pragma unroll
    for (int j = 0; j < 32; j++) t[j] = (colmask >> j) & 1u ? plog2p(g[j] * pscale) : 0.f;
    // segmented sums: t[j] of the first column of each column variable ends
    // up holding the sum over that variable's bins
#pragma unroll
    for (int l = 0; l < LG; l++) {
#pragma unroll
      for (int j = 0; j < 32; j += 2 << l) t[j] += t[j + (1 << l)];
    }
    // ... and over the row variable's bins (its kNb consecutive lanes)
#pragma unroll
    for (int o = kNb >> 1; o > 0; o >>= 1) {
#pragma unroll
      for (int j = 0; j < 32; j += kNb) t[j] += __shfl_xor_sync(0xffffffffu, t[j], o);
    }
    if ((lane & (kNb - 1)) != 0 || x >= nx) return;
    const float hxx = hx[x];
#pragma unroll
    for (int j = 0; j < 32; j += kNb) {
      const int64_t y = (c0 + j) >> LG;
      if (y >= ny || (symmetric && y < x)) continue;
      const float mi = t[j] + hxx + hy[y];
      out[y * ldo + x] = mi;
      if (symmetric && y != x) out[x * ldo + y] = mi;
    }
  }
  __device__ void begin_tile(int64_t, EpiCtx &) const {}
  __device__ void end_tile(EpiCtx &) const {}
  __device__ void drain(EpiCtx &) const {}
};

// Plain FP32 store of the contraction, C[r*ld + c]; with row and column
// scales (operands scaled per row by powers of two), C[r][c] * rs[r] * cs[c].
struct StoreFinish {
  float *out;
  int64_t ld, nr, nc;
  const float *rs = nullptr, *cs = nullptr;
  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], EpiCtx &ctx) const {
    const int lane = threadIdx.x & 31;
    float *wsm = ctx.wsm;
#pragma unroll
    for (int j = 0; j < 32; j++) wsm[lane * 33 + j] = g[j];
    __syncwarp();
    const int64_t rbase = r - lane, c = c0 + lane;
    const float csc = (rs && c < nc) ? cs[c] : 1.f;
    if (rbase + 31 < nr && c0 + 31 < nc) {
      float *o = out + (rbase * ld + c);
      if (rs) {
#pragma unroll 8
        for (int i = 0; i < 32; i++) {
          *o = (wsm[i * 33 + lane] * rs[rbase + i]) * csc;
          o += ld;
        }
      } else {
#pragma unroll 8
        for (int i = 0; i < 32; i++) {
          *o = wsm[i * 33 + lane];
          o += ld;
        }
      }
      __syncwarp();
      return;
    }
    for (int i = 0; i < 32; i++) {
      const int64_t ri = rbase + i;
      if (ri >= nr) break;
      if (c < nc) out[ri * ld + c] = rs ? (wsm[i * 33 + lane] * rs[ri]) * csc : wsm[i * 33 + lane];
    }
    __syncwarp();
  }
  __device__ void begin_tile(int64_t, EpiCtx &) const {}
  __device__ void end_tile(EpiCtx &) const {}
  __device__ void drain(EpiCtx &) const {}
};

// ----------------------------------------------------------------- kernel
// LISTS: the unchunked (Euclidean) kernel, whose epilogue is latency-bound:
// 16 epilogue warps of 64 columns, each with a pending-pair list and its
// columns' norms in shared memory.  The chunked kernels keep 8 warps of 128
// columns (their running sums need the registers) and give the shared
// memory to the stages.
// WIDE: sixteen epilogue warps of 64 columns for a chunked kernel (the
// Pearson finish, whose stores are latency-bound at two warps per scheduler).
template <int KIND, int BK, bool LISTS, bool WIDE = false>
struct TcCfg {
  static constexpr int NSPLIT = tc::Kind<KIND>::NSPLIT;
  static constexpr int EPI = (LISTS || WIDE) ? 16 : 8;       // epilogue warps
  static constexpr int THREADS = 64 + 32 * EPI;              // + producer and MMA warps
  static constexpr int COLS = 4 * kBN / EPI;                 // columns per epilogue warp
  static constexpr int ROW_BYTES = BK * 2;                // 128 or 64
  static constexpr int A_TILE = kBM * BK * 2;
  static constexpr int B_TILE = kBN * BK * 2;
  static constexpr int STAGE = NSPLIT * (A_TILE + B_TILE);
  static constexpr int EPI_FLOATS = kEpiTileFloats + (LISTS ? kEuclidList + 2 * COLS : 0);
  static constexpr int EPI_BYTES = EPI * EPI_FLOATS * 4;
  static constexpr int STAGES_RAW = (kMaxSmem - 1024 - 256 - EPI_BYTES) / STAGE;
  static constexpr int STAGES = STAGES_RAW > 6 ? 6 : STAGES_RAW;
  static constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 256 /*barriers*/ + EPI_BYTES;
  static constexpr int KSTEPS = BK / 16;
  static constexpr int NPROD = NSPLIT == 2 ? 3 : 6;
  static_assert(STAGES >= 2, "need at least two stages");
};

template <int NSPLIT>
__device__ __forceinline__ void product_parts(int p, int &pa, int &pb) {
  // pairs (i, j) with i + j <= NSPLIT - 1, smallest terms first
  if (NSPLIT == 2) {
    const int A[3] = {1, 0, 0}, B[3] = {0, 1, 0};
    pa = A[p]; pb = B[p];
  } else {
    const int A[6] = {2, 1, 0, 1, 0, 0}, B[6] = {0, 1, 2, 0, 1, 0};
    pa = A[p]; pb = B[p];
  }
}

// The dist layout in aligned lines (DistLines, LineTiles): the tiles' origins
// come from a table, so that a lookup is one load the cursor issues a tile
// ahead.
struct EuclidLineWork {
  CUtensorMap ma, mb;
  int64_t nk;
  int64_t ntiles;
  const int2 *tiles;  // (row0, col0) per tile, line_tile_table_kernel
  EuclidLineFinish fin;
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
  __device__ bool skip() const { return false; }
  __device__ const EuclidLineFinish &finish(const TileRef &) const { return fin; }
  __device__ void drain(EpiCtx &ctx) const { fin.drain(ctx); }
  __device__ void prefetch() const {
    tc::prefetch_tensormap(&ma);
    tc::prefetch_tensormap(&mb);
  }
};

// Block I (columns 32 I .. 32 I + 31) of a lane's running sums into the
// warp's staging tile, row = lane.
template <int I, int N>
__device__ __forceinline__ void stage_block(const float (&acc)[N], float *wsm) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < 32; j++) wsm[lane * 33 + j] = acc[32 * I + j];
}

// The finish a work source applies.
template <class Work>
using FinOf = std::decay_t<decltype(std::declval<const Work &>().finish(std::declval<const TileRef &>()))>;

// One contraction whose K range is cut into `parts` pieces, so that a
// contraction of few output tiles still occupies the SMs: work item u is
// output tile u / parts over the k-blocks of piece u % parts, stored by
// fins[piece] (each piece into its own partial output).
template <class Fin>
struct KSplitWork {
  static constexpr int kMaxParts = 4;
  CUtensorMap ma, mb;
  TileSpace ts;
  int64_t nk_total, nk_part;
  int parts;
  Fin fins[kMaxParts];
  __device__ bool tile(int64_t cursor, TileRef &ref) const {
    const int64_t u = int64_t(blockIdx.x) + cursor * int64_t(gridDim.x);
    if (u >= ts.ntiles * parts) return false;
    const int64_t t = u / parts;
    const int64_t piece = u - t * parts;
    int64_t ti, tj;
    tile_coords(ts, t, ti, tj);
    ref.row0 = ti * kBM;
    ref.col0 = tj * kBN;
    ref.ma = &ma;
    ref.mb = &mb;
    ref.k0 = piece * nk_part;
    ref.nk = nk_total - ref.k0 < nk_part ? nk_total - ref.k0 : nk_part;
    ref.prob = piece;
    return true;
  }
  static constexpr bool kPrefetch = false;
  __device__ bool skip() const { return false; }
  __device__ const Fin &finish(const TileRef &ref) const { return fins[ref.prob]; }
  __device__ void drain(EpiCtx &ctx) const { fins[0].drain(ctx); }
  __device__ void prefetch() const {
    tc::prefetch_tensormap(&ma);
    tc::prefetch_tensormap(&mb);
  }
};

// Whether a work source asks for sixteen epilogue warps (Work::kWideEpi).
template <class Work, class = void>
struct wide_epi : std::false_type {};
template <class Work>
struct wide_epi<Work, std::void_t<decltype(Work::kWideEpi)>>
    : std::integral_constant<bool, Work::kWideEpi> {};

// The configuration a kernel runs: chunked kernels whose work source asks for
// it and whose finish takes staged blocks run sixteen epilogue warps where the
// shared memory allows it (32-wide K blocks).  Batches ask for it: their
// outputs are pitched, and on sector-aligned rows the extra warps hide the
// store latency (single problems with a row stride off the 32-byte sectors
// store slower with them).
template <int KIND, int BK, bool CHUNKED, class Work>
using KernelCfg = TcCfg<KIND, BK, !CHUNKED,
                        CHUNKED && BK == 32 && wide_epi<Work>::value &&
                            staged_block<FinOf<Work>>::value>;

template <int KIND, int BK, bool CHUNKED, class Work>
__global__ void __launch_bounds__(KernelCfg<KIND, BK, CHUNKED, Work>::THREADS, 1)
gram_tc_kernel(const __grid_constant__ Work work, int64_t ckb, const tc::WaitCfg wc) {
  using C = KernelCfg<KIND, BK, CHUNKED, Work>;
  if (work.skip()) return;  // a gated launch whose gate is closed: before any setup
  constexpr int NSPLIT = C::NSPLIT;
  static_assert(!CHUNKED || C::COLS == 128 || C::COLS == 64,
                "chunked sums hold 128 or 64 columns per warp");
  static_assert(CHUNKED || C::COLS == kEuclidCols, "the list kernels hold 64 columns per warp");
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + C::STAGES * C::STAGE);
  uint64_t *empty = full + C::STAGES;
  uint64_t *accf = empty + C::STAGES;
  uint64_t *acce = accf + 2;
  uint64_t *mma_done = acce + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  float *epi_smem = reinterpret_cast<float *>(smem + C::STAGES * C::STAGE + 256);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      tc::mbar_init(&accf[b], 1);
      tc::mbar_init(&acce[b], C::EPI);
    }
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_barrier_init();
  }
  if (warp == 0 && lane == 0) work.prefetch();
  if (warp == 1) tc::tmem_alloc(tmem_slot, 2 * kBN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------ TMA producer
      int64_t it = 0;
      TileRef ref;
      TileCursor<Work> tiles(work, 0, 1);
      while (!*abort_flag && tiles.next(ref)) {
        for (int64_t kb = 0; kb < ref.nk; kb++, it++) {
          const int s = int(it % C::STAGES);
          const uint32_t use = uint32_t(it / C::STAGES);
          if (!tc::mbar_wait(&empty[s], (use & 1u) ^ 1u, abort_flag, wc)) {
            *abort_flag = 1;
            break;
          }
          uint8_t *st = smem + s * C::STAGE;
          tc::mbar_arrive_expect_tx(&full[s], C::STAGE);
#pragma unroll
          for (int p = 0; p < NSPLIT; p++)
            tc::tma_load_3d(st + p * C::A_TILE, ref.ma, &full[s], int32_t((ref.k0 + kb) * BK),
                            int32_t(ref.row0), p);
#pragma unroll
          for (int p = 0; p < NSPLIT; p++)
            tc::tma_load_3d(st + NSPLIT * C::A_TILE + p * C::B_TILE, ref.mb, &full[s],
                            int32_t((ref.k0 + kb) * BK), int32_t(ref.col0), p);
        }
      }
      // drain: no bulk copy may still be writing shared memory at exit
      if (*abort_flag) {
        for (int s = 0; s < C::STAGES; s++) {
          const int64_t fills = it / C::STAGES + (s < it % C::STAGES ? 1 : 0);
          if (fills > 0) tc::mbar_wait_bounded(&full[s], uint32_t((fills - 1) & 1), kDrainLimitNs);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------ MMA issuer
      constexpr uint32_t idesc = tc::idesc_f32acc(kBM, kBN, tc::Kind<KIND>::AB_FMT);
      int64_t it = 0, cc = 0;
      bool ok = true;
      TileRef ref;
      TileCursor<Work> tiles(work, 0, 1);
      while (ok && tiles.next(ref)) {
        const int64_t ck = CHUNKED ? ckb : ref.nk;
        const int64_t nch = (ref.nk + ck - 1) / ck;
        for (int64_t ch = 0; ch < nch && ok; ch++, cc++) {
          const int buf = int(cc & 1);
          const uint32_t ause = uint32_t(cc >> 1);
          if (!tc::mbar_wait(&acce[buf], (ause & 1u) ^ 1u, abort_flag, wc)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t d = tmem_base + uint32_t(buf * kBN);
          const int64_t kb0 = ch * ck, kb1 = (kb0 + ck < ref.nk) ? kb0 + ck : ref.nk;
          for (int64_t kb = kb0; kb < kb1; kb++, it++) {
            const int s = int(it % C::STAGES);
            const uint32_t use = uint32_t(it / C::STAGES);
            if (!tc::mbar_wait(&full[s], use & 1u, abort_flag, wc)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(smem + s * C::STAGE);
            const uint32_t sb = sa + NSPLIT * C::A_TILE;
#pragma unroll
            for (int k = 0; k < C::KSTEPS; k++) {
#pragma unroll
              for (int p = 0; p < C::NPROD; p++) {
                int pa, pb;
                product_parts<NSPLIT>(p, pa, pb);
                const uint64_t ad = tc::smem_desc_kmajor(sa + pa * C::A_TILE + k * 32, C::ROW_BYTES);
                const uint64_t bd = tc::smem_desc_kmajor(sb + pb * C::B_TILE + k * 32, C::ROW_BYTES);
                tc::umma_bf16(d, ad, bd, idesc, (kb != kb0 || k || p) ? 1u : 0u);
              }
            }
            tc::umma_commit(&empty[s]);
          }
          if (ok) tc::umma_commit(&accf[buf]);
        }
      }
      if (!ok) *abort_flag = 1;
      // every MMA issued above has finished before TMEM is released
      tc::umma_commit(mma_done);
      tc::mbar_wait_bounded(mma_done, 0u, kDrainLimitNs);
    }
    __syncwarp();
  } else {
    // ------------------------------------------ epilogue (warps 2..9)
    const int q = warp & 3;            // TMEM lane quarter
    const int part = (warp - 2) >> 2;  // column part: 0 .. EPI/4 - 1
    EpiCtx ctx;
    float *mine = epi_smem + (warp - 2) * C::EPI_FLOATS;
    ctx.wsm = mine;
    ctx.nlist = 0;
    ctx.gcount = 0;
    int64_t cc = 0;  // accumulator use counter: buffer cc & 1, phase cc >> 1
    bool ok = true;
    TileRef ref;
    TileCursor<Work> tiles(work, 0, 1);
    while (ok && tiles.next(ref)) {
      const auto &fin = work.finish(ref);
      const int64_t r = ref.row0 + q * 32 + lane;
      const int64_t col = ref.col0 + part * C::COLS;
      ctx.rbase = r - lane;
      ctx.col0 = col;
      fin.begin_tile(r, ctx);
      if constexpr (CHUNKED) {
        const int64_t nch = (ref.nk + ckb - 1) / ckb;
        float acc[C::COLS];
#pragma unroll
        for (int j = 0; j < C::COLS; j++) acc[j] = 0.f;
        for (int64_t ch = 0; ch < nch; ch++, cc++) {
          const int buf = int(cc & 1);
          const uint32_t ause = uint32_t(cc >> 1);
          const bool got = tc::mbar_wait(&accf[buf], ause & 1u, abort_flag, wc);
          if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t tb =
              tmem_base + uint32_t(buf * kBN + part * C::COLS) + (uint32_t(q * 32) << 16);
#pragma unroll
          for (int i = 0; i < C::COLS / 16; i++) {
            float g[16];
            tc::tmem_ld16(tb + uint32_t(16 * i), g);
#pragma unroll
            for (int j = 0; j < 16; j++) acc[16 * i + j] += g[j];
          }
          tc::tc_fence_before();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&acce[buf]);
        }
        if (!ok) break;
        using FinT = std::decay_t<decltype(fin)>;
        if constexpr (staged_block<FinT>::value) {
          // One copy of the finish for the four 32-column blocks, each staged
          // in the warp's tile first: four inlined copies outgrow the
          // instruction cache once the epilogue bounds the kernel (small n).
#pragma unroll 1
          for (int i = 0; i < C::COLS / 32; i++) {
            if (!fin.block_live(r - lane, col + 32 * i)) continue;
            if constexpr (C::COLS == 64) {
              if (i == 0) stage_block<0>(acc, ctx.wsm);
              else stage_block<1>(acc, ctx.wsm);
            } else {
              switch (i) {
                case 0: stage_block<0>(acc, ctx.wsm); break;
                case 1: stage_block<1>(acc, ctx.wsm); break;
                case 2: stage_block<2>(acc, ctx.wsm); break;
                default: stage_block<3>(acc, ctx.wsm); break;
              }
            }
            __syncwarp();
            fin.block(r, col + 32 * i, ctx);
          }
        } else {
#pragma unroll
          for (int i = 0; i < C::COLS / 32; i++) {
            float g[32];
#pragma unroll
            for (int j = 0; j < 32; j++) g[j] = acc[32 * i + j];
            fin(r, col + 32 * i, g, ctx);
          }
        }
        fin.end_tile(ctx);
      } else {
        const int buf = int(cc & 1);
        const uint32_t ause = uint32_t(cc >> 1);
        const bool got = tc::mbar_wait(&accf[buf], ause & 1u, abort_flag, wc);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t tb =
            tmem_base + uint32_t(buf * kBN + part * C::COLS) + (uint32_t(q * 32) << 16);
#pragma unroll 1
        for (int i = 0; i < C::COLS / 32; i++) {
          float g[32];
          tc::tmem_ld32(tb + uint32_t(32 * i), g);
          fin(r, col + 32 * i, g, ctx);
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&acce[buf]);
        cc++;
        fin.end_tile(ctx);
      }
    }
    if (ok) work.drain(ctx);  // pairs that wait across tiles
    if (!ok) *abort_flag = 1;
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) atomicOr(wc.err, 1);
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_base, 2 * kBN);
  }
}

// ----------------------------------------------------------------- operands
// Split planes of one row (a variable or a point): parts of val(k) for
// k < n, zeros for n <= k < kpad; four consecutive k per lane, stored as one
// 8-byte word per plane.  `plane` is the element stride between part planes.
template <int KIND, class Val>
__device__ __forceinline__ void write_row_planes(int64_t n, int64_t kpad, int64_t plane,
                                                 uint16_t *__restrict__ z, Val &&val) {
  constexpr int NS = tc::Kind<KIND>::NSPLIT;
  const int lane = threadIdx.x & 31;
  for (int64_t k0 = 4 * int64_t(lane); k0 < kpad; k0 += 128) {
    uint32_t w[3][2];
#pragma unroll
    for (int q = 0; q < 3; q++) w[q][0] = w[q][1] = 0u;
    if (k0 < n) {
      float v[4];
      val(k0, v);
#pragma unroll
      for (int e = 0; e < 4; e++) {
        uint16_t p[3];
        tc::split_parts<KIND>(v[e], p);
        if (k0 + e >= n) p[0] = p[1] = p[2] = 0;
#pragma unroll
        for (int q = 0; q < 3; q++) w[q][e >> 1] |= uint32_t(p[q]) << (16 * (e & 1));
      }
    }
#pragma unroll
    for (int q = 0; q < NS; q++)
      *reinterpret_cast<uint2 *>(z + q * plane + k0) = make_uint2(w[q][0], w[q][1]);
  }
}

// Pearson planes of variable x (length n) with statistics s: z = (x - mean) *
// inv_norm (times 2^14 for f16x3), NaN for every k < n of a NaN-flagged or
// constant variable.
template <int KIND>
__device__ __forceinline__ void pearson_row(const float *__restrict__ x, int64_t n, int64_t kpad,
                                            int64_t plane, const ColStats &s,
                                            uint16_t *__restrict__ z) {
  const Centerer cen(s);
  const float scale = tc::Kind<KIND>::F16 ? 16384.f : 1.f;
  const bool nanrow = s.flags != 0;
  const bool vec = (reinterpret_cast<uintptr_t>(x) & 15u) == 0 && (n & 3) == 0;
  write_row_planes<KIND>(n, kpad, plane, z, [&](int64_t k0, float (&v)[4]) {
    if (vec) {
      const float4 t = *reinterpret_cast<const float4 *>(x + k0);
      v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else {
#pragma unroll
      for (int e = 0; e < 4; e++) v[e] = (k0 + e < n) ? x[k0 + e] : 0.f;
    }
#pragma unroll
    for (int e = 0; e < 4; e++) v[e] = nanrow ? __int_as_float(0x7fc00000) : cen(v[e]) * scale;
  });
}

// Pearson prologue, fused: one warp per variable computes the statistics and
// writes the operand planes (and the statistics, when st is not null).
template <int KIND>
__global__ void __launch_bounds__(256)
pearson_prep_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int64_t kpad,
                    uint16_t *__restrict__ Z, ColStats *__restrict__ st) {
  const int64_t v = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (v >= nvar) return;  // whole warps
  const float *x = X + v * n;
  const ColStats s = colstats_warp(x, n, GT_EVERYTHING);
  if (st && (threadIdx.x & 31) == 0) st[v] = s;
  pearson_row<KIND>(x, n, kpad, nvar * kpad, s, Z + v * kpad);
}

// Column sums of the points: block (x, y) sums dimensions 32x .. 32x+31 over
// points 64y .. 64y+63 (8 rows of 32 lanes, compensated float sums, combined
// in a fixed order), one partial per (point block, dimension).
constexpr int kColsumPoints = 64;
__global__ void __launch_bounds__(256)
euclid_colsum_kernel(const float *__restrict__ P, int64_t n, int64_t dim,
                     double *__restrict__ partial) {
  __shared__ float2 sh[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t d = int64_t(blockIdx.x) * 32 + tx;
  const int64_t i0 = int64_t(blockIdx.y) * kColsumPoints;
  FloatPairSum acc;
  if (d < dim) {
#pragma unroll 8
    for (int i = ty; i < kColsumPoints; i += 8)
      if (i0 + i < n) acc.add(P[(i0 + i) * dim + d]);
  }
  sh[ty][tx] = make_float2(acc.hi, acc.lo);
  __syncthreads();
  if (ty == 0 && d < dim) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < 8; r++) s += double(sh[r][tx].x) + double(sh[r][tx].y);
    partial[blockIdx.y * dim + d] = s;
  }
}

// Column means as float pairs (hi, lo): one CTA per dimension sums that
// dimension's partials (strided per thread, then a fixed tree), so the
// result does not depend on scheduling.
__global__ void __launch_bounds__(256)
euclid_mean_kernel(const double *__restrict__ partial, int64_t nblk, int64_t dim, int64_t n,
                   float2 *__restrict__ mean2) {
  __shared__ double sh[256];
  const int64_t d = blockIdx.x;
  double s = 0.0;
  for (int64_t b = threadIdx.x; b < nblk; b += 256) s += partial[b * dim + d];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = sh[0] / double(n);
    const float hi = float(m);
    mean2[d] = make_float2(hi, float(m - double(hi)));
  }
}

// Euclidean operand planes of the centred points, one warp per point: the
// squared norm (compensated), the largest magnitude (f16x3 scale), then the
// planes.  nrm[v] = {|c|^2, 2^-s}; rows n .. npad-1 of nrm are zeroed.  With
// ZB, the planes also go to row lines.pos(v) of the permuted column operand
// (npb rows), whose padding rows are zeroed, and the column tables of the
// aligned-lines finish are written.
template <int KIND>
__global__ void __launch_bounds__(256)
euclid_split_kernel(const float *__restrict__ P, int64_t n, int64_t npad, int64_t dim,
                    int64_t kpad, const float2 *__restrict__ mean2, uint16_t *__restrict__ Z,
                    float2 *__restrict__ nrm, uint16_t *__restrict__ ZB, int64_t npb,
                    const DistLines lines, int4 *__restrict__ colinfo,
                    int64_t *__restrict__ groupbase) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int64_t plane = n * kpad, planeB = npb * kpad;
  const int64_t nslot = npad > npb ? npad : npb;
  for (int64_t v = warp; v < nslot; v += nwarps) {
    // padding rows of the permuted column operand are zero, their column
    // entries the sentinel point n
    if (ZB && v < npb && lines.point(v) >= n) {
      write_row_planes<KIND>(0, kpad, planeB, ZB + v * kpad, [](int64_t, float (&)[4]) {});
      if (lane == 0) {
        colinfo[v] = make_int4(int(n), 0, 0, 0);
        if ((v % EuclidLineFinish::kCols) == 0) groupbase[v / EuclidLineFinish::kCols] = 0;
      }
    }
    if (v >= n) {
      if (v < npad && lane == 0) nrm[v] = make_float2(0.f, 0.f);
      continue;
    }
    const float *x = P + v * dim;
    FloatPairSum acc;
    float res = 0.f, amax = 0.f;
    for (int64_t k = lane; k < dim; k += 32) {
      const float2 m = mean2[k];
      const float c = (x[k] - m.x) - m.y;
      const float q = c * c;
      res += fmaf(c, c, -q);
      acc.add(q);
      amax = fmaxf(amax, fabsf(c));
    }
    float hi = acc.hi, lo = acc.lo + res;
    warp_pair_sum(hi, lo);
    amax = __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(amax)));
    const int se = tc::Kind<KIND>::F16 ? tc::f16_scale_exp(amax) : 0;
    const float scale = tc::exp2i(se);
    if (lane == 0) nrm[v] = make_float2(hi + lo, tc::exp2i(-se));
    auto val = [&](int64_t k0, float (&c)[4]) {
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int64_t k = k0 + e;
        if (k < dim) {
          const float2 m = mean2[k];
          c[e] = ((x[k] - m.x) - m.y) * scale;
        } else {
          c[e] = 0.f;
        }
      }
    };
    write_row_planes<KIND>(dim, kpad, plane, Z + v * kpad, val);
    if (ZB) {
      const int64_t p = lines.pos(v);
      write_row_planes<KIND>(dim, kpad, planeB, ZB + p * kpad, val);
      if (lane == 0) {
        // the dist column base of v, relative to its column group's first
        // point (the group's smallest)
        constexpr int64_t G = EuclidLineFinish::kCols;
        const int64_t c0 = lines.point(p / G * G);
        const int64_t b = n * v - v * (v + 1) / 2 - v - 1;
        const int64_t b0 = n * c0 - c0 * (c0 + 1) / 2 - c0 - 1;
        colinfo[p] = make_int4(int(v), int(b - b0), __float_as_int(hi + lo),
                               __float_as_int(tc::exp2i(-se)));
        if (p % G == 0) groupbase[p / G] = b0;
      }
    }
  }
}

// (row0, col0) of every aligned-lines tile.
__global__ void __launch_bounds__(256)
line_tile_table_kernel(const LineTiles lt, int2 *__restrict__ tab) {
  const uint32_t u = blockIdx.x * 256u + threadIdx.x;
  if (u >= lt.ntiles) return;
  int64_t r0, c0;
  lt.decode(u, r0, c0);
  tab[u] = make_int2(int(r0), int(c0));
}

// Exact distances of the near-zero pairs the aligned-lines Gram kernel
// listed: block r takes region r (counts[r] pairs (row, column), row >
// column) and overwrites their dist entries, 64 pairs per round (4 lanes
// each).  Every lane issues all its coordinate loads of a batch before the
// first use, and the next round's entries load during this round.  Runs
// after the Gram kernel on the same stream.
constexpr int kFixupThreads = 256;
__global__ void __launch_bounds__(kFixupThreads)
euclid_fixup_kernel(const float *__restrict__ pts, int64_t n, int64_t dim, int vec4,
                    float *__restrict__ out, const int2 *__restrict__ pairs,
                    const int *__restrict__ counts, int cap) {
  constexpr int PER_ROUND = kFixupThreads / 4;
  const unsigned FULLM = 0xffffffffu;
  const int sub = threadIdx.x & 3, slot = threadIdx.x >> 2;
  const int2 *list = pairs + int64_t(blockIdx.x) * cap;
  int cnt = counts[blockIdx.x];
  cnt = cnt < 0 ? 0 : (cnt > cap ? cap : cnt);
  if (cnt == 0) return;
  int2 e = list[slot < cnt ? slot : 0];
  for (int b = 0; b < cnt; b += PER_ROUND) {
    const bool act = b + slot < cnt;
    const int nb = b + PER_ROUND;
    const int2 en = nb + slot < cnt ? list[nb + slot] : e;
    const bool ok = act && e.y >= 0 && e.y < e.x && int64_t(e.x) < n;
    const int64_t i = ok ? e.x : 0, j = ok ? e.y : 0;
    const float *pa = pts + i * dim, *pb = pts + j * dim;
    FloatPairSum acc;
    float res = 0.f;
    if (vec4) {
      const float4 *a4 = reinterpret_cast<const float4 *>(pa);
      const float4 *b4 = reinterpret_cast<const float4 *>(pb);
      const int64_t d4 = dim >> 2;
      for (int64_t k0 = sub; k0 < d4; k0 += 32) {
        float4 x[8], y[8];
#pragma unroll
        for (int it = 0; it < 8; it++) {
          const int64_t k = k0 + 4 * it;
          x[it] = k < d4 ? a4[k] : make_float4(0.f, 0.f, 0.f, 0.f);
          y[it] = k < d4 ? b4[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int it = 0; it < 8; it++) {
          sq_add(x[it].x - y[it].x, acc, res);
          sq_add(x[it].y - y[it].y, acc, res);
          sq_add(x[it].z - y[it].z, acc, res);
          sq_add(x[it].w - y[it].w, acc, res);
        }
      }
    } else {
      for (int64_t k = sub; k < dim; k += 4) sq_add(pa[k] - pb[k], acc, res);
    }
    float hi = acc.hi, lo = acc.lo + res;
#pragma unroll
    for (int o = 2; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(FULLM, hi, o), ol = __shfl_xor_sync(FULLM, lo, o);
      const float t = hi + oh, bp = t - hi;
      lo = (lo + ol) + ((hi - (t - bp)) + (oh - bp));
      hi = t;
    }
    if (ok && sub == 0) out[n * j - j * (j + 1) / 2 - j - 1 + i] = sqrtf(hi + lo);
    e = en;
  }
}

// Batched Pearson prologue: the variables of every problem, one warp each.
struct PearsonBatchInput {
  const float *X;
  int64_t p, n, kpad;
  int64_t plane_off;  // element offset of this problem's planes (NSPLIT x p x kpad)
  int64_t var_off;    // offset of its variables in the global variable index
};

template <int KIND>
__global__ void __launch_bounds__(256)
pearson_batch_prep_kernel(const PearsonBatchInput *__restrict__ in,
                          const int64_t *__restrict__ var_prefix, int64_t nprob,
                          int64_t total_vars, uint16_t *__restrict__ planes) {
  const int64_t gv = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (gv >= total_vars) return;  // whole warps
  const int64_t pi = find_segment(var_prefix, nprob, gv);
  const PearsonBatchInput b = in[pi];
  const int64_t v = gv - var_prefix[pi];
  const float *x = b.X + v * b.n;
  const ColStats s = colstats_warp(x, b.n, GT_EVERYTHING);
  pearson_row<KIND>(x, b.n, b.kpad, b.p * b.kpad, s, planes + b.plane_off + v * b.kpad);
}

// ----------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 3-D map over planes [nsplit][rows][kpad] of 16-bit parts; box {bk, box_rows, 1}.
int make_plane_map(CUtensorMap *map, const void *base, int64_t rows, int64_t kpad, int nsplit,
                   int box_rows, int bk, bool f16) {
  auto fn = encode_fn();
  if (!fn) return fail(GT_ECUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {cuuint64_t(kpad), cuuint64_t(rows), cuuint64_t(nsplit)};
  cuuint64_t strides[2] = {cuuint64_t(kpad * 2), cuuint64_t(rows * kpad * 2)};
  cuuint32_t box[3] = {cuuint32_t(bk), cuuint32_t(box_rows), 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = fn(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                  const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(GT_ECUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
  return GT_OK;
}

// Launches the persistent kernel over `ntiles` tiles of work source w.
template <int KIND, int BK, bool CHUNKED, class W>
int launch_work(const W &w, int64_t ntiles, int64_t ckb, const char *prof_name,
                cudaStream_t s) {
  using C = KernelCfg<KIND, BK, CHUNKED, W>;
  if (ntiles == 0) return GT_OK;
  tc::WaitCfg wc;
  GT_TRY(make_wait_cfg(&wc));
  auto kern = gram_tc_kernel<KIND, BK, CHUNKED, W>;
  GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
  const int64_t grid = ntiles < sm_count() ? ntiles : sm_count();
  ProfScope prof(prof_name, s);
  kern<<<unsigned(grid), C::THREADS, C::SMEM, s>>>(w, ckb, wc);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

template <int KIND, int BK, bool CHUNKED, class Fin>
int launch_gram(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                int mode, int64_t ckb, const Fin &fin, const char *prof_name,
                cudaStream_t s) {
  using C = TcCfg<KIND, BK, !CHUNKED>;
  using W = SingleWork<Fin>;
  constexpr bool F16 = tc::Kind<KIND>::F16;
  if (kpad <= 0 || kpad % BK) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  if (ckb < 1) ckb = 1;
  W w;
  GT_TRY(make_plane_map(&w.ma, zA, nA, kpad, C::NSPLIT, kBM, BK, F16));
  GT_TRY(make_plane_map(&w.mb, zB, nB, kpad, C::NSPLIT, kBN, BK, F16));
  w.ts = make_tiles(nA, nB, mode, band_group(int64_t(kBN) * kpad * 2 * C::NSPLIT));
  if (w.ts.ntiles > 2147483647LL) return fail(GT_EINVAL, "problem too large (%lld tiles)",
                                             (long long)w.ts.ntiles);
  w.nk = kpad / BK;
  w.fin = fin;
  return launch_work<KIND, BK, CHUNKED>(w, w.ts.ntiles, ckb, prof_name, s);
}

// Pending near-zero pairs per epilogue warp that the aligned-lines kernel
// lists for euclid_fixup_kernel (8 KB x 8 per warp); beyond them a warp
// recomputes its pairs itself.
constexpr int64_t kPairCap = 8192;

// The aligned-lines tiling pays about 8192 / n extra tiles on the diagonal;
// it is used from 32768 points on (GT_EUCLID_LINES=1 / 0 forces it on / off).
bool use_dist_lines(int64_t n) {
  const char *e = std::getenv("GT_EUCLID_LINES");
  if (e && *e) return std::atoi(e) != 0;
  return n >= 32768;
}

int tc_config() {
  static int cfg = -1;
  if (cfg < 0) {
    const char *e = std::getenv("GT_TC_BK");
    cfg = (e && std::atoi(e) == 64) ? 64 : 32;
  }
  return cfg;
}

// k-blocks per accumulation chunk of the Pearson contraction (GT_TC_CHUNK
// elements, default 256; 0 = a single chunk).
int64_t tc_chunk_kblocks(int bk) {
  static int64_t elems = -1;
  if (elems < 0) {
    const char *e = std::getenv("GT_TC_CHUNK");
    elems = e ? std::atoll(e) : 256;
  }
  if (elems <= 0) return int64_t(1) << 40;
  return elems / bk > 0 ? elems / bk : 1;
}

int check_kind(int kind) {
  if (kind != tc::KIND_BF16X3 && kind != tc::KIND_BF16X6 && kind != tc::KIND_F16X3)
    return fail(GT_EINVAL, "not a tensor-core split (%d)", kind);
  return GT_OK;
}

int kind_nsplit(int kind) { return kind == tc::KIND_BF16X6 ? 3 : 2; }

}  // namespace

int tc_plane_map(CUtensorMap *map, const void *base, int64_t rows, int64_t kpad, int nplanes,
                 int box_rows, int bk, bool f16) {
  return make_plane_map(map, base, rows, kpad, nplanes, box_rows, bk, f16);
}

// Mutual information from f16x3 weight planes (rows = variable * 2^lg + bin,
// each weight times 2^14): the chunked Gram with MiFinish.
int mi_tc(const void *planesX, int64_t rowsX, const void *planesY, int64_t rowsY, int64_t kpad,
          int lg, int nbins, int64_t nx, int64_t ny, int64_t nsamples, const float *hx,
          const float *hy, float *out, int symmetric, cudaStream_t s) {
  if (rowsX == 0 || rowsY == 0) return GT_OK;
  unsigned colmask = 0u;
  for (int j = 0; j < 32; j++)
    if ((j & ((1 << lg) - 1)) < nbins) colmask |= 1u << j;
  const float pscale = float(1.0 / (268435456.0 * double(nsamples)));
  // FP32 chunks of 512 samples: 15 % faster than 256 at 10 bins x 1000 samples, with a
  // largest MI error of 7.5e-6 bits against the FP64 oracle (4.1e-6 with 256)
  auto run = [&](auto lgc) {
    constexpr int LG = decltype(lgc)::value;
    MiFinish<LG> fin{out, hx, hy, nx, ny, nx, pscale, symmetric, colmask};
    return launch_gram<tc::KIND_F16X3, 32, true>(planesX, rowsX, planesY, rowsY, kpad,
                                                 symmetric ? kUpper : kFull, 512 / 32, fin,
                                                 "mi_gram", s);
  };
  switch (lg) {
    case 0: return run(std::integral_constant<int, 0>{});
    case 1: return run(std::integral_constant<int, 1>{});
    case 2: return run(std::integral_constant<int, 2>{});
    case 3: return run(std::integral_constant<int, 3>{});
    case 4: return run(std::integral_constant<int, 4>{});
    case 5: return run(std::integral_constant<int, 5>{});
    default: return fail(GT_EINVAL, "bins beyond the tensor-core path (%d)", 1 << lg);
  }
}

// C[r][c] = sum_k A_r[k] B_c[k] over split-bf16 planes ([part][row][kpad]),
// chunked FP32 accumulation, stored as a row-major float matrix.
int gemm_tc_store(const void *planesA, int64_t nA, const void *planesB, int64_t nB, int64_t kpad,
                  int nsplit, float *C, int64_t ldc, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  StoreFinish fin{C, ldc, nA, nB};
  if (nsplit == 3)
    return launch_gram<tc::KIND_BF16X6, 32, true>(planesA, nA, planesB, nB, kpad, kFull,
                                                  tc_chunk_kblocks(32), fin, "gemm_store", s);
  return launch_gram<tc::KIND_BF16X3, 64, true>(planesA, nA, planesB, nB, kpad, kFull,
                                                tc_chunk_kblocks(64), fin, "gemm_store", s);
}

// C_q = A B^T over the q-th of up to `parts` pieces of the K range (bf16x6
// planes), each piece into C + q * nA * ldc, all in one launch (the caller
// adds the pieces); parts is at most 4, every piece gets at least one k-block,
// and *used says how many pieces were written.
int gemm_tc_store_ksplit(const void *planesA, int64_t nA, const void *planesB, int64_t nB,
                         int64_t kpad, int parts, int *used, float *C, int64_t ldc,
                         cudaStream_t s) {
  *used = 0;
  if (nA == 0 || nB == 0) return GT_OK;
  using W = KSplitWork<StoreFinish>;
  constexpr int BK = 32;
  if (kpad <= 0 || kpad % BK) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  const int64_t nk = kpad / BK;
  if (parts < 1 || parts > W::kMaxParts) return fail(GT_EINVAL, "bad K split (%d)", parts);
  if (parts > nk) parts = int(nk);
  W w;
  GT_TRY(make_plane_map(&w.ma, planesA, nA, kpad, 3, kBM, BK, false));
  GT_TRY(make_plane_map(&w.mb, planesB, nB, kpad, 3, kBN, BK, false));
  w.ts = make_tiles(nA, nB, kFull, band_group(int64_t(kBN) * kpad * 2 * 3));
  w.nk_total = nk;
  w.nk_part = cdiv(nk, int64_t(parts));
  w.parts = int(cdiv(nk, w.nk_part));  // every piece non-empty
  for (int q = 0; q < w.parts; q++)
    w.fins[q] = StoreFinish{C + int64_t(q) * nA * ldc, ldc, nA, nB};
  *used = w.parts;
  return launch_work<tc::KIND_BF16X6, BK, true>(w, w.ts.ntiles * w.parts, tc_chunk_kblocks(BK),
                                                "gemm_store", s);
}

// The same contraction from f16x3 planes whose rows were scaled by powers of
// two (rsA, rsB: the factors 2^-e that undo each row's scale).
int gemm_tc_store_scaled(const void *planesA, int64_t nA, const void *planesB, int64_t nB,
                         int64_t kpad, const float *rsA, const float *rsB, float *C, int64_t ldc,
                         cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  StoreFinish fin{C, ldc, nA, nB, rsA, rsB};
  return launch_gram<tc::KIND_F16X3, 32, true>(planesA, nA, planesB, nB, kpad, kFull,
                                               tc_chunk_kblocks(32), fin, "gemm_store", s);
}

int pearson_tc_prologue(const float *dX, int64_t nvar, int64_t n, int kind, int slot_z,
                        int slot_st, void **Z, int64_t *kpad, cudaStream_t s) {
  if (kind == tc::KIND_F16X6) return pearson_exact_prologue(dX, nvar, n, slot_z, Z, kpad, s);
  GT_TRY(check_kind(kind));
  *kpad = cdiv(n, kKPad) * kKPad;
  void *pz = nullptr, *pst = nullptr;
  GT_TRY(ws_get(slot_z, size_t(kind_nsplit(kind)) * size_t(nvar) * size_t(*kpad) * 2, &pz));
  GT_TRY(ws_get(slot_st, size_t(nvar) * sizeof(ColStats), &pst));
  auto *st = static_cast<ColStats *>(pst);
  auto *z = static_cast<uint16_t *>(pz);
  const int64_t blocks = cdiv(nvar, 8);
  if (blocks > 2147483647LL) return fail(GT_EINVAL, "too many variables");
  ProfScope prof("pearson_prologue", s);
  if (kind == tc::KIND_BF16X6)
    pearson_prep_kernel<tc::KIND_BF16X6><<<unsigned(blocks), 256, 0, s>>>(dX, nvar, n, *kpad, z, st);
  else if (kind == tc::KIND_F16X3)
    pearson_prep_kernel<tc::KIND_F16X3><<<unsigned(blocks), 256, 0, s>>>(dX, nvar, n, *kpad, z, st);
  else
    pearson_prep_kernel<tc::KIND_BF16X3><<<unsigned(blocks), 256, 0, s>>>(dX, nvar, n, *kpad, z, st);
  count_launch();
  GT_CUDA(cudaGetLastError());
  *Z = pz;
  return GT_OK;
}

int pearson_tc(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad, int kind,
               const PearsonOut &out, cudaStream_t s) {
  if (kind == tc::KIND_F16X6) return pearson_exact(zA, nA, zB, nB, kpad, out, s);
  GT_TRY(check_kind(kind));
  if (nA == 0 || nB == 0) return GT_OK;
  if (!out.corr && !out.ts && !out.pairs) return GT_OK;
  const float gscale = kind == tc::KIND_F16X3 ? 1.f / 268435456.f : 1.f;  // 2^-28
  PearsonFinish fin{out.corr, out.ts, out.pairs, out.ld, nA, nB, out.npairs,
                    std::sqrt(out.npairs - 2.f), gscale, out.symmetric};
  fin.gate = out.gate;
  const int sym = out.symmetric ? kUpper : kFull;
  if (kind == tc::KIND_BF16X6)
    return launch_gram<tc::KIND_BF16X6, 32, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(32),
                                                  fin, "pearson_gram", s);
  if (kind == tc::KIND_F16X3) {
    if (tc_config() == 32)
      return launch_gram<tc::KIND_F16X3, 32, true>(zA, nA, zB, nB, kpad, sym,
                                                   tc_chunk_kblocks(32), fin, "pearson_gram", s);
    return launch_gram<tc::KIND_F16X3, 64, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(64),
                                                 fin, "pearson_gram", s);
  }
  if (tc_config() == 32)
    return launch_gram<tc::KIND_BF16X3, 32, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(32),
                                                  fin, "pearson_gram", s);
  return launch_gram<tc::KIND_BF16X3, 64, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(64),
                                                fin, "pearson_gram", s);
}

void pearson_band_tiles(int64_t nr, int64_t nc, bool symmetric, int64_t band_blocks,
                        std::vector<int2> &tiles, std::vector<int64_t> &offsets) {
  band_tiles(nr, nc, symmetric, band_blocks, tiles, offsets);
}

// The Pearson Gram on the tiles tiles[0 .. ntiles) (device table of
// (row0, col0), band_tiles): f16x3 (k-block 32) and f16x6 only.
int pearson_tc_band(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad, int kind,
                    const PearsonOut &out, const int2 *tiles, int64_t ntiles, cudaStream_t s) {
  if (kind == tc::KIND_F16X6) return pearson_exact_band(zA, nA, zB, nB, kpad, out, tiles, ntiles, s);
  if (kind != tc::KIND_F16X3) return fail(GT_EUNSUPPORTED, "banded Gram: f16x3 and f16x6 only");
  if (ntiles == 0) return GT_OK;
  using W = TableWork<PearsonFinish>;
  W w;
  GT_TRY(make_plane_map(&w.ma, zA, nA, kpad, 2, kBM, 32, true));
  GT_TRY(make_plane_map(&w.mb, zB, nB, kpad, 2, kBN, 32, true));
  w.tiles = tiles;
  w.ntiles = ntiles;
  w.nk = kpad / 32;
  w.fin = PearsonFinish{out.corr, out.ts, out.pairs, out.ld, nA, nB, out.npairs,
                        std::sqrt(out.npairs - 2.f), 1.f / 268435456.f, out.symmetric};
  w.fin.gate = out.gate;
  return launch_work<tc::KIND_F16X3, 32, true>(w, ntiles, tc_chunk_kblocks(32), "pearson_gram", s);
}

namespace {

template <int KIND>
int euclid_tc_kind(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
                   float tau, cudaStream_t st) {
  constexpr int NS = tc::Kind<KIND>::NSPLIT;
  constexpr bool F16 = tc::Kind<KIND>::F16;
  const int64_t kpad = cdiv(dim, kKPad) * kKPad;
  const int64_t npad = cdiv(n, kBN) * kBN;
  const int64_t nblk = cdiv(n, kColsumPoints);
  DistLines lines{};
  LineTiles lt{};
  const bool aligned = layout == GT_LAYOUT_DIST && use_dist_lines(n) &&
                       make_dist_lines(n, reinterpret_cast<uintptr_t>(d_out), &lines) &&
                       make_line_tiles(n, &lt);
  // permuted column operand of the aligned lines: 8192 rows per super-block
  const int64_t npb = aligned ? lt.npb : 0;
  void *pz = nullptr, *pn = nullptr, *pp = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, size_t(NS) * size_t(n + npb) * size_t(kpad) * 2, &pz));
  // nrm, then (aligned lines) the column tables and the tile table
  const size_t nrm_bytes = size_t(npad) * sizeof(float2);
  const size_t ci_bytes = size_t(npb) * sizeof(int4);
  const size_t gb_bytes = size_t(npb / EuclidLineFinish::kCols) * 8;
  const size_t tab_bytes = aligned ? size_t(lt.ntiles) * sizeof(int2) : 0;
  GT_TRY(ws_get(WS_SCRATCH2, nrm_bytes + ci_bytes + gb_bytes + tab_bytes, &pn));
  auto *colinfo = reinterpret_cast<int4 *>(static_cast<char *>(pn) + nrm_bytes);
  auto *groupbase = reinterpret_cast<int64_t *>(static_cast<char *>(pn) + nrm_bytes + ci_bytes);
  auto *tiletab =
      reinterpret_cast<int2 *>(static_cast<char *>(pn) + nrm_bytes + ci_bytes + gb_bytes);
  GT_TRY(ws_get(WS_SCRATCH3, size_t(nblk) * size_t(dim) * 8 + size_t(dim) * sizeof(float2), &pp));
  auto *z = static_cast<uint16_t *>(pz);
  auto *zb = aligned ? z + size_t(NS) * size_t(n) * size_t(kpad) : nullptr;
  auto *nrm = static_cast<float2 *>(pn);
  auto *partial = static_cast<double *>(pp);
  auto *mean2 = reinterpret_cast<float2 *>(partial + nblk * dim);
  {
    ProfScope prof("euclid_prologue", st);
    if (nblk > 65535) return fail(GT_EINVAL, "too many points (%lld)", (long long)n);
    dim3 cg((unsigned)cdiv(dim, 32), (unsigned)nblk, 1u);
    euclid_colsum_kernel<<<cg, 256, 0, st>>>(d_pts, n, dim, partial);
    euclid_mean_kernel<<<unsigned(dim), 256, 0, st>>>(partial, nblk, dim, n, mean2);
    const int64_t slots = npad > npb ? npad : npb;
    int64_t g = cdiv(slots * 32, 256);
    if (g > int64_t(sm_count()) * 16) g = int64_t(sm_count()) * 16;
    euclid_split_kernel<KIND><<<unsigned(g), 256, 0, st>>>(d_pts, n, npad, dim, kpad, mean2, z,
                                                           nrm, zb, npb, lines, colinfo,
                                                           groupbase);
    count_launch(3);
    if (aligned) {
      line_tile_table_kernel<<<unsigned(cdiv(int64_t(lt.ntiles), 256)), 256, 0, st>>>(lt, tiletab);
      count_launch();
    }
    GT_CUDA(cudaGetLastError());
  }
  const int vec4 = (reinterpret_cast<uintptr_t>(d_pts) & 15u) == 0 && (dim & 3) == 0;
  if (!aligned) {
    EuclidFinish fin{nrm, d_pts, d_out, n, dim, layout, tau, vec4};
    return launch_gram<KIND, 32, false>(z, n, z, n, kpad, kLower, 0, fin, "euclid_gram", st);
  }
  using C = TcCfg<KIND, 32, true>;
  const int64_t grid = int64_t(lt.ntiles) < sm_count() ? int64_t(lt.ntiles) : sm_count();
  const int64_t regions = grid * C::EPI;
  void *pl = nullptr;
  GT_TRY(ws_get(WS_SCRATCH1, size_t(regions) * (size_t(kPairCap) * sizeof(int2) + sizeof(int)), &pl));
  auto *pairs = static_cast<int2 *>(pl);
  auto *counts = reinterpret_cast<int *>(pairs + regions * kPairCap);
  GT_CUDA(cudaMemsetAsync(counts, 0, size_t(regions) * sizeof(int), st));
  EuclidLineWork w;
  GT_TRY(make_plane_map(&w.ma, z, n, kpad, NS, kBM, 32, F16));
  GT_TRY(make_plane_map(&w.mb, zb, npb, kpad, NS, kBN, 32, F16));
  w.nk = kpad / 32;
  w.ntiles = int64_t(lt.ntiles);
  w.tiles = tiletab;
  w.fin = EuclidLineFinish{nrm, colinfo, groupbase, d_pts, d_out, n, dim, tau, vec4, pairs,
                           counts, int(kPairCap), C::EPI};
  GT_TRY((launch_work<KIND, 32, false>(w, int64_t(lt.ntiles), 0, "euclid_gram", st)));
  ProfScope prof("euclid_fixup", st);
  euclid_fixup_kernel<<<unsigned(regions), kFixupThreads, 0, st>>>(d_pts, n, dim, vec4, d_out, pairs, counts,
                                                        int(kPairCap));
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace

int euclid_tc(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
              cudaStream_t st) {
  if (dim == 0 || n < 2) return dist_simt(d_pts, n, dim, d_out, layout, GT_EUCLIDEAN, 2.f, st);
  // The 3-product split of bf16 loses too much for distances, so the bf16
  // paths use bf16x6.  Entries with d^2 below tau (|a|^2 + |b|^2) are
  // recomputed exactly: tau = 1/8 for bf16x6 (float32-level products), 1/4
  // for f16x3 (~2^-21 products).
  // (the exact Pearson setting, f16x6, runs distances as f16x3: with the
  // near-zero recomputation they already meet its precision)
  const int path = gt_get_gram_path();
  if (path == GT_GRAM_TC_F16X3 || path == GT_GRAM_TC_F16X6)
    return euclid_tc_kind<tc::KIND_F16X3>(d_pts, n, dim, d_out, layout, 0.25f, st);
  return euclid_tc_kind<tc::KIND_BF16X6>(d_pts, n, dim, d_out, layout, 0.125f, st);
}

// Batched cor(x): builds device descriptors (through `alloc`, which the plan
// owns), balances the tiles over one CTA per SM, and returns the runner that
// launches prologue + Gram for the whole batch.
int pearson_batch_prepare(const gt_cor_problem *probs, int64_t count, int kind, int bk,
                          int64_t chunk_elems, const std::function<int(size_t, void **)> &alloc,
                          std::function<int(cudaStream_t)> *run, int64_t *ntiles_out,
                          int64_t *nctas_out, int **err_out) {
  GT_TRY(check_kind(kind));
  if (bk != 32 && bk != 64) return fail(GT_EINVAL, "bad k-block (%d)", bk);
  if (kind == tc::KIND_BF16X6) bk = 32;
  const int nsplit = kind_nsplit(kind);
  const bool f16 = kind == tc::KIND_F16X3;
  std::vector<PearsonBatchInput> inputs;
  std::vector<PearsonBatchProblem> descs;
  std::vector<int64_t> var_prefix{0}, tile_prefix{0}, cost;
  std::vector<int4> table_all;  // {problem, row0, col0, k-blocks} per global tile
  int64_t plane_elems = 0, vars = 0;
  // first pass: shapes and offsets
  for (int64_t i = 0; i < count; i++) {
    const gt_cor_problem &q = probs[i];
    if (q.p < 0 || q.n < 0) return fail(GT_EINVAL, "problem %lld: negative size", (long long)i);
    if (q.p == 0) continue;
    if (!q.X) return fail(GT_EINVAL, "problem %lld: null input", (long long)i);
    if (q.n == 0) return fail(GT_EINVAL, "problem %lld: no observations", (long long)i);
    if (q.ld != 0 && q.ld < q.p)
      return fail(GT_EINVAL, "problem %lld: output row stride %lld below p", (long long)i,
                  (long long)q.ld);
    PearsonBatchInput b;
    b.X = q.X;
    b.p = q.p;
    b.n = q.n;
    b.kpad = cdiv(q.n, kKPad) * kKPad;
    b.plane_off = plane_elems;
    b.var_off = vars;
    inputs.push_back(b);
    plane_elems += int64_t(nsplit) * b.p * b.kpad;
    vars += b.p;
    var_prefix.push_back(vars);
  }
  const int64_t nprob = int64_t(inputs.size());
  void *d_planes = nullptr, *d_in = nullptr, *d_vp = nullptr;
  GT_TRY(alloc(size_t(plane_elems) * 2, &d_planes));
  auto *planes = static_cast<uint16_t *>(d_planes);
  int64_t ckb = chunk_elems / bk;
  if (ckb < 1) ckb = 1;
  const float gscale = f16 ? 1.f / 268435456.f : 1.f;
  // second pass: tensor maps, tiles, finishes
  int64_t pidx = 0;
  for (int64_t i = 0; i < count; i++) {
    const gt_cor_problem &q = probs[i];
    if (q.p == 0) continue;
    const PearsonBatchInput &b = inputs[pidx++];
    PearsonBatchProblem d{};  // value-initialised: zero bytes, padding included
    GT_TRY(make_plane_map(&d.map_a, planes + b.plane_off, b.p, b.kpad, nsplit, kBM, bk, f16));
    GT_TRY(make_plane_map(&d.map_b, planes + b.plane_off, b.p, b.kpad, nsplit, kBN, bk, f16));
    d.ts = make_tiles(b.p, b.p, kUpper, band_group(int64_t(kBN) * b.kpad * 2 * nsplit));
    d.nk = b.kpad / bk;
    d.fin = PearsonFinish{q.corr, q.ts, q.pairs, q.ld != 0 ? q.ld : b.p, b.p, b.p, float(b.n),
                          std::sqrt(float(b.n) - 2.f), gscale, 1};
    descs.push_back(d);
    tile_prefix.push_back(tile_prefix.back() + d.ts.ntiles);
    // Cost of a tile (ns, on one SM): its MMAs, or its epilogue when that
    // takes longer -- tiles of few observations are bound by their stores
    // (12 bytes per entry and orientation, ~24 bytes per ns per SM measured
    // on single problems) -- plus a fixed part per tile.
    const int64_t prods = nsplit == 3 ? 6 : 3;
    const double mma_ns = double(d.nk) * (bk / 16) * prods * 128.0 / 1.9;
    for (int64_t t = 0; t < d.ts.ntiles; t++) {
      int64_t ti, tj;
      tile_coords(d.ts, t, ti, tj);
      const int64_t r0 = ti * kBM, r1 = std::min(b.p, r0 + kBM);
      const int64_t c0 = tj * kBN, c1 = std::min(b.p, c0 + kBN);
      int64_t upper = 0, diag = 0;
      for (int64_t r = r0; r < r1; r++) {
        upper += std::max<int64_t>(0, c1 - std::max(c0, r));
        diag += (r >= c0 && r < c1) ? 1 : 0;
      }
      const double epi_ns = 12.0 * double(2 * upper - diag) / 24.0;
      cost.push_back(int64_t(std::max(mma_ns, epi_ns) + 1500.0));
      table_all.push_back(make_int4(int(pidx - 1), int(r0), int(c0), int(d.nk)));
    }
  }
  const int64_t ntiles = tile_prefix.back();
  int64_t ncta = sm_count();
  if (ncta > ntiles) ncta = ntiles;
  std::vector<int4> cta_tiles;
  std::vector<int64_t> cta_off;
  if (ntiles > 0) {
    // list scheduling in an order that keeps operand panels shared: the
    // problems by decreasing total cost, each problem's tiles in its band
    // order, every tile to the CTA with the least work so far -- so the CTAs
    // running at one time work on neighbouring tiles of one problem and read
    // its panels from L2 (a longest-tile-first order spread every problem over
    // the whole run)
    std::vector<int64_t> porder(descs.size());
    std::vector<int64_t> pcost(descs.size(), 0);
    for (size_t q = 0; q < descs.size(); q++) {
      porder[q] = int64_t(q);
      for (int64_t t = tile_prefix[q]; t < tile_prefix[q + 1]; t++) pcost[q] += cost[t];
    }
    std::stable_sort(porder.begin(), porder.end(),
                     [&](int64_t a, int64_t c) { return pcost[a] > pcost[c]; });
    std::vector<int64_t> order;
    order.reserve(size_t(ntiles));
    for (int64_t q : porder)
      for (int64_t t = tile_prefix[q]; t < tile_prefix[q + 1]; t++) order.push_back(t);
    std::vector<std::vector<int64_t>> lists(ncta);
    using Item = std::pair<int64_t, int64_t>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (int64_t c = 0; c < ncta; c++) heap.push({0, c});
    for (int64_t t : order) {
      Item it = heap.top();
      heap.pop();
      lists[it.second].push_back(t);
      it.first += cost[t];
      heap.push(it);
    }
    cta_off.assign(ncta + 1, 0);
    for (int64_t c = 0; c < ncta; c++) {
      cta_off[c] = int64_t(cta_tiles.size());
      for (int64_t t : lists[c]) cta_tiles.push_back(table_all[t]);
    }
    cta_off[ncta] = int64_t(cta_tiles.size());
  }
  auto upload = [&](const void *src, size_t bytes, void **dst) -> int {
    GT_TRY(alloc(bytes, dst));
    if (bytes) GT_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return GT_OK;
  };
  void *d_desc = nullptr, *d_ct = nullptr, *d_co = nullptr;
  GT_TRY(upload(inputs.data(), inputs.size() * sizeof(PearsonBatchInput), &d_in));
  GT_TRY(upload(var_prefix.data(), var_prefix.size() * 8, &d_vp));
  GT_TRY(upload(descs.data(), descs.size() * sizeof(PearsonBatchProblem), &d_desc));
  GT_TRY(upload(cta_tiles.data(), cta_tiles.size() * sizeof(int4), &d_ct));
  GT_TRY(upload(cta_off.data(), cta_off.size() * 8, &d_co));
  // the device's error word; the wait limit is the one in force when the plan is built
  tc::WaitCfg wc;
  GT_TRY(make_wait_cfg(&wc));
  PearsonBatchWork w;
  w.probs = static_cast<const PearsonBatchProblem *>(d_desc);
  w.table = static_cast<const int4 *>(d_ct);
  w.cta_off = static_cast<const int64_t *>(d_co);
  auto *in = static_cast<const PearsonBatchInput *>(d_in);
  auto *vp = static_cast<const int64_t *>(d_vp);
  *err_out = wc.err;
  const int64_t total_vars = vars;
  const int BKc = bk;
  *ntiles_out = ntiles;
  *nctas_out = ncta;
  *run = [=](cudaStream_t s) -> int {
    if (total_vars == 0) return GT_OK;
    const int64_t blocks = cdiv(total_vars, 8);
    if (blocks > 2147483647LL) return fail(GT_EINVAL, "too many variables in the batch");
    if (kind == tc::KIND_BF16X6)
      pearson_batch_prep_kernel<tc::KIND_BF16X6>
          <<<unsigned(blocks), 256, 0, s>>>(in, vp, nprob, total_vars, planes);
    else if (kind == tc::KIND_F16X3)
      pearson_batch_prep_kernel<tc::KIND_F16X3>
          <<<unsigned(blocks), 256, 0, s>>>(in, vp, nprob, total_vars, planes);
    else
      pearson_batch_prep_kernel<tc::KIND_BF16X3>
          <<<unsigned(blocks), 256, 0, s>>>(in, vp, nprob, total_vars, planes);
    count_launch();
    if (ncta == 0) return GT_OK;
    auto launch = [&](auto kern, int threads, int smem) -> int {
      GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      kern<<<unsigned(ncta), threads, smem, s>>>(w, ckb, wc);
      return GT_OK;
    };
    using W = PearsonBatchWork;
    if (kind == tc::KIND_BF16X6) {
      using C = KernelCfg<tc::KIND_BF16X6, 32, true, W>;
      GT_TRY(launch(gram_tc_kernel<tc::KIND_BF16X6, 32, true, W>, C::THREADS, C::SMEM));
    } else if (kind == tc::KIND_F16X3) {
      using C32 = KernelCfg<tc::KIND_F16X3, 32, true, W>;
      using C64 = KernelCfg<tc::KIND_F16X3, 64, true, W>;
      if (BKc == 32)
        GT_TRY(launch(gram_tc_kernel<tc::KIND_F16X3, 32, true, W>, C32::THREADS, C32::SMEM));
      else
        GT_TRY(launch(gram_tc_kernel<tc::KIND_F16X3, 64, true, W>, C64::THREADS, C64::SMEM));
    } else {
      using C32 = KernelCfg<tc::KIND_BF16X3, 32, true, W>;
      using C64 = KernelCfg<tc::KIND_BF16X3, 64, true, W>;
      if (BKc == 32)
        GT_TRY(launch(gram_tc_kernel<tc::KIND_BF16X3, 32, true, W>, C32::THREADS, C32::SMEM));
      else
        GT_TRY(launch(gram_tc_kernel<tc::KIND_BF16X3, 64, true, W>, C64::THREADS, C64::SMEM));
    }
    count_launch();
    GT_CUDA(cudaGetLastError());
    return GT_OK;
  };
  return GT_OK;
}

}  // namespace gt
