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
// z = (x - mean)/||x - mean|| computed in FP64 and rounded to float;
// Euclidean: the centred coordinate) is split into bf16 parts
// v = v0 + v1 [+ v2], each the round-to-nearest bf16 of the remainder of the
// previous ones.  The parts live in separate planes [part][row][k] (K
// contiguous, padded to a multiple of 64 with zeros).  The Gram entry is the
// sum of the part products of total order at most NSPLIT-1:
//   NSPLIT = 2 ("bf16x3"): v0w0 + v0w1 + v1w0            (~2^-16 relative)
//   NSPLIT = 3 ("bf16x6"): + v0w2 + v1w1 + v2w0            (float32-level)
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
#include <vector>

namespace gt {

namespace {

constexpr int kTcThreads = 320;                   // 2 control warps + 8 epilogue warps
constexpr int kEpiWarps = 8;
constexpr int kBM = 128, kBN = 256;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per barrier wait
constexpr uint64_t kDrainLimitNs = 200000000ull;  // 0.2 s for in-flight work at exit
constexpr int kKPad = 64;                         // K padding of the operand planes
constexpr int kMaxSmem = 232448;                  // dynamic shared memory per CTA (227 KB)
constexpr int kEpiTileFloats = 32 * 33;           // one warp's padded 32 x 32 staging tile

// ----------------------------------------------------------------- tiling
struct TileSpace {
  int64_t tr, tc;    // row blocks (128), column blocks (256)
  int64_t j0;        // symmetric: column blocks whose tile count is 2*tj + 2
  int64_t ntiles;
  int symmetric;
};

// Symmetric problems: column block tj holds row blocks 0 .. min(2 tj + 1, tr-1)
// (the 128-row blocks that reach the upper triangle of a 256-column block).
__host__ __device__ inline void tile_coords(const TileSpace &ts, int64_t t, int64_t &ti,
                                            int64_t &tj) {
  if (!ts.symmetric) {
    tj = t / ts.tr;
    ti = t - tj * ts.tr;
    return;
  }
  const int64_t head = ts.j0 * (ts.j0 + 1);
  if (t < head) {
    int64_t j = int64_t((sqrt(4.0 * double(t) + 1.0) - 1.0) * 0.5);
    while ((j + 1) * (j + 2) <= t) j++;
    while (j * (j + 1) > t) j--;
    tj = j;
    ti = t - j * (j + 1);
  } else {
    const int64_t u = t - head;
    tj = ts.j0 + u / ts.tr;
    ti = u - (tj - ts.j0) * ts.tr;
  }
}

TileSpace make_tiles(int64_t nr, int64_t nc, bool symmetric) {
  TileSpace ts;
  ts.tr = cdiv(nr, kBM);
  ts.tc = cdiv(nc, kBN);
  ts.symmetric = symmetric ? 1 : 0;
  if (symmetric) {
    ts.j0 = ts.tr / 2;
    if (ts.j0 > ts.tc) ts.j0 = ts.tc;
    ts.ntiles = ts.j0 * (ts.j0 + 1) + (ts.tc - ts.j0) * ts.tr;
  } else {
    ts.j0 = 0;
    ts.ntiles = ts.tr * ts.tc;
  }
  return ts;
}

// ----------------------------------------------------------------- finishes
// Each finish handles a warp's 32 x 32 block: lane = row r (consecutive rows
// across lanes), g[j] = entry (r, c0 + j); wsm is the warp's staging tile.

__device__ __forceinline__ float clamp_r(float r) { return r > 1.f ? 1.f : (r < -1.f ? -1.f : r); }

// hostSignif's rule (src/correlation.cpp:51-64), t = r sqrt(n-2) / sqrt(1-r^2)
// with sqrt(n-2) precomputed and a hardware reciprocal square root.
__device__ __forceinline__ float signif_fast(float r, float sq_nm2) {
  if (r >= 0.999f) return 10000.0f;
  return r * sq_nm2 * tc::rsqrt_approx(1.f - r * r);
}

struct PearsonFinish {
  float *corr, *ts, *pairs;
  int64_t ld, nr, nc;
  float npairs, sq_nm2;
  int symmetric;

  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], float *wsm) const {
    const int lane = threadIdx.x & 31;
    // mirror orientation (lanes hold consecutive rows): coalesced from registers
    if (symmetric && r < nr) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int64_t c = c0 + j;
        if (c < nc && r < c) {
          const float v = clamp_r(g[j]);
          const int64_t o = c * ld + r;
          if (corr) corr[o] = v;
          if (ts) ts[o] = signif_fast(v, sq_nm2);
          if (pairs) pairs[o] = npairs;
        }
      }
    }
    // row orientation through the staging tile
#pragma unroll
    for (int j = 0; j < 32; j++) wsm[lane * 33 + j] = g[j];
    __syncwarp();
    const int64_t rbase = r - lane;
    const int64_t c = c0 + lane;
    int64_t o = rbase * ld + c;
    for (int i = 0; i < 32; i++, o += ld) {
      const int64_t ri = rbase + i;
      if (ri >= nr) break;
      if (c >= nc || (symmetric && c < ri)) continue;
      float v = clamp_r(wsm[i * 33 + lane]);
      if (symmetric && c == ri && v == v) v = 1.f;
      if (corr) corr[o] = v;
      if (ts) ts[o] = signif_fast(v, sq_nm2);
      if (pairs) pairs[o] = npairs;
    }
    __syncwarp();
  }
};

// Operands are the points centred by their column means (distances do not
// change).  d^2 = |a|^2 + |b|^2 - 2 G with FP32 norms rounded from FP64; an
// entry whose d^2 is below tau * (|a|^2 + |b|^2), where rounding of the
// contraction could dominate, is recomputed from the original float points
// by the warp (float differences and partial sums per lane, FP64 sum across
// lanes), so exact duplicates come out exactly 0.
struct EuclidFinish {
  const float *norm2;
  const float *pts;
  float *out;
  int64_t n, dim;
  int layout;  // GT_LAYOUT_FULL / GT_LAYOUT_DIST
  float tau;

  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], float *wsm) const {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t cl = c0 + lane;
    const float nbl = cl < n ? norm2[cl] : 0.f;
    const float na = r < n ? norm2[r] : 0.f;
    // this lane's row uses columns c0 + j with r < c0 + j < n
    const int64_t lo64 = r + 1 - c0, hi64 = n - c0;
    const int jlo = lo64 < 0 ? 0 : (lo64 > 32 ? 32 : int(lo64));
    const int jhi = r >= n ? 0 : (hi64 > 32 ? 32 : (hi64 < 0 ? 0 : int(hi64)));
    float v[32];
    unsigned pend = 0u;
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const float s = na + __shfl_sync(FULL, nbl, j);
      const float d2 = fmaf(-2.f, g[j], s);
      const bool valid = (j >= jlo) & (j < jhi);
      pend |= unsigned(valid & (d2 < tau * s)) << j;
      v[j] = valid ? tc::sqrt_approx(fmaxf(d2, 0.f)) : 0.f;
    }
    while (true) {
      const unsigned any = __ballot_sync(FULL, pend != 0u);
      if (!any) break;
      const int src = __ffs(int(any)) - 1;
      const int j = __shfl_sync(FULL, __ffs(int(pend)) - 1, src);
      const long long rr = __shfl_sync(FULL, (long long)r, src);
      const float *pa = pts + rr * dim, *pb = pts + (c0 + j) * dim;
      float part = 0.f;
      for (int64_t k = lane; k < dim; k += 32) {
        const float d = pa[k] - pb[k];
        part = fmaf(d, d, part);
      }
      double acc = double(part);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
      if (lane == src) {
        const float d = sqrtf(float(acc));
#pragma unroll
        for (int q = 0; q < 32; q++)
          if (q == j) v[q] = d;
        pend &= ~(1u << j);
      }
    }
    const bool full = layout == GT_LAYOUT_FULL;
    if (full && r < n) {
#pragma unroll
      for (int j = 0; j < 32; j++)
        if (j >= jlo && j < jhi) out[(c0 + j) * n + r] = v[j];
    }
#pragma unroll
    for (int j = 0; j < 32; j++) wsm[lane * 33 + j] = v[j];
    __syncwarp();
    const int64_t rbase = r - lane, c = c0 + lane;
    // offset of (row rbase, column 0): full n*r; R dist n*r - r(r+1)/2 - r - 1
    int64_t off = full ? rbase * n : n * rbase - rbase * (rbase + 1) / 2 - rbase - 1;
    for (int i = 0; i < 32; i++) {
      const int64_t ri = rbase + i;
      if (ri >= n) break;
      if (c < n) {
        if (full) {
          if (c >= ri) out[off + c] = (c == ri) ? 0.f : wsm[i * 33 + lane];
        } else if (c > ri) {
          out[off + c] = wsm[i * 33 + lane];
        }
      }
      off += full ? n : n - ri - 2;
    }
    __syncwarp();
  }
};

// Plain FP32 store of the contraction, C[r*ld + c].
struct StoreFinish {
  float *out;
  int64_t ld, nr, nc;
  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32], float *wsm) const {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < 32; j++) wsm[lane * 33 + j] = g[j];
    __syncwarp();
    const int64_t rbase = r - lane, c = c0 + lane;
    for (int i = 0; i < 32; i++) {
      const int64_t ri = rbase + i;
      if (ri >= nr) break;
      if (c < nc) out[ri * ld + c] = wsm[i * 33 + lane];
    }
    __syncwarp();
  }
};

// ----------------------------------------------------------------- kernel
template <int NSPLIT, int BK>
struct TcCfg {
  static constexpr int ROW_BYTES = BK * 2;                // 128 or 64
  static constexpr int A_TILE = kBM * BK * 2;
  static constexpr int B_TILE = kBN * BK * 2;
  static constexpr int STAGE = NSPLIT * (A_TILE + B_TILE);
  static constexpr int EPI_BYTES = kEpiWarps * kEpiTileFloats * 4;
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

// ----------------------------------------------------------------- work sources
// A work source tells every role of the kernel, for the cursor-th tile of
// this CTA, which tensor maps to load from, the tile's row / column blocks,
// its number of k-blocks, and the finish to apply.
struct TileRef {
  const CUtensorMap *ma, *mb;
  int64_t ti, tj, nk, prob;
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
    tile_coords(ts, t, ref.ti, ref.tj);
    ref.ma = &ma;
    ref.mb = &mb;
    ref.nk = nk;
    ref.prob = 0;
    return true;
  }
  __device__ const Fin &finish(const TileRef &) const { return fin; }
  __device__ void prefetch() const {
    tc::prefetch_tensormap(&ma);
    tc::prefetch_tensormap(&mb);
  }
};

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
struct alignas(64) PearsonBatchProblem {
  CUtensorMap map;
  TileSpace ts;
  int64_t nk;
  PearsonFinish fin;
};

struct PearsonBatchWork {
  const PearsonBatchProblem *probs;
  const int64_t *tile_prefix;
  int64_t nprob;
  const int64_t *cta_tiles, *cta_off;
  __device__ bool tile(int64_t cursor, TileRef &ref) const {
    const int64_t idx = cta_off[blockIdx.x] + cursor;
    if (idx >= cta_off[blockIdx.x + 1]) return false;
    const int64_t t = cta_tiles[idx];
    const int64_t pi = find_segment(tile_prefix, nprob, t);
    const PearsonBatchProblem &pr = probs[pi];
    tile_coords(pr.ts, t - tile_prefix[pi], ref.ti, ref.tj);
    ref.ma = ref.mb = &pr.map;
    ref.nk = pr.nk;
    ref.prob = pi;
    return true;
  }
  __device__ PearsonFinish finish(const TileRef &ref) const { return probs[ref.prob].fin; }
  __device__ void prefetch() const {}
};

template <int NSPLIT, int BK, bool CHUNKED, class Work>
__global__ void __launch_bounds__(kTcThreads, 1)
gram_tc_kernel(const __grid_constant__ Work work, int64_t ckb, int *err) {
  using C = TcCfg<NSPLIT, BK>;
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
      tc::mbar_init(&acce[b], kEpiWarps);
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
      for (int64_t cur = 0; !*abort_flag && work.tile(cur, ref); cur++) {
        for (int64_t kb = 0; kb < ref.nk; kb++, it++) {
          const int s = int(it % C::STAGES);
          const uint32_t use = uint32_t(it / C::STAGES);
          if (!tc::mbar_wait(&empty[s], (use & 1u) ^ 1u, abort_flag, kWaitLimitNs)) {
            *abort_flag = 1;
            break;
          }
          uint8_t *st = smem + s * C::STAGE;
          tc::mbar_arrive_expect_tx(&full[s], C::STAGE);
#pragma unroll
          for (int p = 0; p < NSPLIT; p++)
            tc::tma_load_3d(st + p * C::A_TILE, ref.ma, &full[s], int32_t(kb * BK),
                            int32_t(ref.ti * kBM), p);
#pragma unroll
          for (int p = 0; p < NSPLIT; p++)
            tc::tma_load_3d(st + NSPLIT * C::A_TILE + p * C::B_TILE, ref.mb, &full[s],
                            int32_t(kb * BK), int32_t(ref.tj * kBN), p);
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
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN);
      int64_t it = 0, cc = 0;
      bool ok = true;
      TileRef ref;
      for (int64_t cur = 0; ok && work.tile(cur, ref); cur++) {
        const int64_t ck = CHUNKED ? ckb : ref.nk;
        const int64_t nch = (ref.nk + ck - 1) / ck;
        for (int64_t ch = 0; ch < nch && ok; ch++, cc++) {
          const int buf = int(cc & 1);
          const uint32_t ause = uint32_t(cc >> 1);
          if (!tc::mbar_wait(&acce[buf], (ause & 1u) ^ 1u, abort_flag, kWaitLimitNs)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t d = tmem_base + uint32_t(buf * kBN);
          const int64_t kb0 = ch * ck, kb1 = (kb0 + ck < ref.nk) ? kb0 + ck : ref.nk;
          for (int64_t kb = kb0; kb < kb1; kb++, it++) {
            const int s = int(it % C::STAGES);
            const uint32_t use = uint32_t(it / C::STAGES);
            if (!tc::mbar_wait(&full[s], use & 1u, abort_flag, kWaitLimitNs)) {
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
    const int half = (warp - 2) >> 2;  // column half: 0 or 1
    float *wsm = epi_smem + (warp - 2) * kEpiTileFloats;
    int64_t cc = 0;
    bool ok = true;
    TileRef ref;
    for (int64_t cur = 0; ok && work.tile(cur, ref); cur++) {
      const auto fin = work.finish(ref);
      const int64_t r = ref.ti * kBM + q * 32 + lane;
      const int64_t col = ref.tj * kBN + half * 128;
      if (CHUNKED) {
        const int64_t nch = (ref.nk + ckb - 1) / ckb;
        float acc[128];
#pragma unroll
        for (int j = 0; j < 128; j++) acc[j] = 0.f;
        for (int64_t ch = 0; ch < nch; ch++, cc++) {
          const int buf = int(cc & 1);
          const uint32_t ause = uint32_t(cc >> 1);
          const bool got = tc::mbar_wait(&accf[buf], ause & 1u, abort_flag, kWaitLimitNs);
          if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t tb =
              tmem_base + uint32_t(buf * kBN + half * 128) + (uint32_t(q * 32) << 16);
#pragma unroll
          for (int i = 0; i < 8; i++) {
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
#pragma unroll
        for (int i = 0; i < 4; i++) {
          float g[32];
#pragma unroll
          for (int j = 0; j < 32; j++) g[j] = acc[32 * i + j];
          fin(r, col + 32 * i, g, wsm);
        }
      } else {
        const int buf = int(cc & 1);
        const uint32_t ause = uint32_t(cc >> 1);
        const bool got = tc::mbar_wait(&accf[buf], ause & 1u, abort_flag, kWaitLimitNs);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t tb = tmem_base + uint32_t(buf * kBN + half * 128) + (uint32_t(q * 32) << 16);
#pragma unroll 1
        for (int i = 0; i < 4; i++) {
          float g[32];
          tc::tmem_ld32(tb + uint32_t(32 * i), g);
          fin(r, col + 32 * i, g, wsm);
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&acce[buf]);
        cc++;
      }
    }
    if (!ok) *abort_flag = 1;
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) atomicExch(err, 1);
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_base, 2 * kBN);
  }
}

// ----------------------------------------------------------------- operands
// Pearson operand planes: z = (x - mean) * inv_norm in FP64 (rounded to
// float), NaN rows for variables that are NaN-flagged or constant; k >= n is
// zero.  One CTA per variable (no per-element index division).
template <int NSPLIT>
__global__ void __launch_bounds__(256)
pearson_split_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int64_t kpad,
                     const ColStats *__restrict__ st, __nv_bfloat16 *__restrict__ Z) {
  const int64_t v = blockIdx.x;
  const int64_t plane = nvar * kpad;
  const ColStats s = st[v];
  const float *x = X + v * n;
  __nv_bfloat16 *z = Z + v * kpad;
  for (int64_t k = threadIdx.x; k < kpad; k += blockDim.x) {
    __nv_bfloat16 p[3];
    if (k >= n) {
      p[0] = p[1] = p[2] = __float2bfloat16(0.f);
    } else if (s.flags) {
      p[0] = p[1] = p[2] = __float2bfloat16(__int_as_float(0x7fc00000));
    } else {
      tc::split_bf16<NSPLIT>(float((double(x[k]) - s.mean) * s.inv_norm), p);
    }
#pragma unroll
    for (int q = 0; q < NSPLIT; q++) z[q * plane + k] = p[q];
  }
}

// Column sums of the points (FP64), accumulated into sums[] (zeroed first).
__global__ void euclid_colsum_kernel(const float *__restrict__ P, int64_t n, int64_t dim,
                                     int64_t per_block, double *__restrict__ sums) {
  const int64_t d = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (d >= dim) return;
  const int64_t i0 = blockIdx.y * per_block;
  const int64_t i1 = min(n, i0 + per_block);
  double acc = 0.0;
  for (int64_t i = i0; i < i1; i++) acc += double(P[i * dim + d]);
  atomicAdd(&sums[d], acc);
}

// Euclidean operand planes of the centred points and their squared norms
// (FP64, stored rounded to float), one warp per point.
template <int NSPLIT>
__global__ void euclid_split_kernel(const float *__restrict__ P, int64_t n, int64_t dim,
                                    int64_t kpad, const double *__restrict__ sums,
                                    __nv_bfloat16 *__restrict__ Z, float *__restrict__ norm2) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int64_t plane = n * kpad;
  const double inv_n = 1.0 / double(n);
  for (int64_t v = warp; v < n; v += nwarps) {
    double acc = 0.0;
    for (int64_t k = lane; k < kpad; k += 32) {
      __nv_bfloat16 p[3];
      if (k < dim) {
        const double x = double(P[v * dim + k]) - sums[k] * inv_n;
        acc = fma(x, x, acc);
        tc::split_bf16<NSPLIT>(float(x), p);
      } else {
        p[0] = p[1] = p[2] = __float2bfloat16(0.f);
      }
#pragma unroll
      for (int q = 0; q < NSPLIT; q++) Z[q * plane + v * kpad + k] = p[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) norm2[v] = float(acc);
  }
}

// Batched Pearson prologue: the variables of every problem, one CTA each.
struct PearsonBatchInput {
  const float *X;
  int64_t p, n, kpad;
  int64_t plane_off;  // element offset of this problem's planes (NSPLIT x p x kpad)
  int64_t var_off;    // offset of its variables in the statistics array
};

__global__ void __launch_bounds__(kColStatThreads)
pearson_batch_stats_kernel(const PearsonBatchInput *__restrict__ in,
                           const int64_t *__restrict__ var_prefix, int64_t nprob,
                           ColStats *__restrict__ st) {
  __shared__ double sh[32];
  const int64_t gv = blockIdx.x;
  const int64_t pi = find_segment(var_prefix, nprob, gv);
  const PearsonBatchInput b = in[pi];
  const int64_t v = gv - var_prefix[pi];
  const ColStats c = colstats_block(b.X + v * b.n, b.n, GT_EVERYTHING, sh);
  if (threadIdx.x == 0) st[gv] = c;
}

template <int NSPLIT>
__global__ void __launch_bounds__(256)
pearson_batch_split_kernel(const PearsonBatchInput *__restrict__ in,
                           const int64_t *__restrict__ var_prefix, int64_t nprob,
                           const ColStats *__restrict__ st, __nv_bfloat16 *__restrict__ planes) {
  const int64_t gv = blockIdx.x;
  const int64_t pi = find_segment(var_prefix, nprob, gv);
  const PearsonBatchInput b = in[pi];
  const int64_t v = gv - var_prefix[pi];
  const ColStats s = st[gv];
  const int64_t plane = b.p * b.kpad;
  const float *x = b.X + v * b.n;
  __nv_bfloat16 *z = planes + b.plane_off + v * b.kpad;
  for (int64_t k = threadIdx.x; k < b.kpad; k += blockDim.x) {
    __nv_bfloat16 p[3];
    if (k >= b.n) {
      p[0] = p[1] = p[2] = __float2bfloat16(0.f);
    } else if (s.flags) {
      p[0] = p[1] = p[2] = __float2bfloat16(__int_as_float(0x7fc00000));
    } else {
      tc::split_bf16<NSPLIT>(float((double(x[k]) - s.mean) * s.inv_norm), p);
    }
#pragma unroll
    for (int q = 0; q < NSPLIT; q++) z[q * plane + k] = p[q];
  }
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

// 3-D map over planes [nsplit][rows][kpad] of bf16; box {bk, box_rows, 1}.
int make_plane_map(CUtensorMap *map, const void *base, int64_t rows, int64_t kpad, int nsplit,
                   int box_rows, int bk) {
  auto fn = encode_fn();
  if (!fn) return fail(GT_ECUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {cuuint64_t(kpad), cuuint64_t(rows), cuuint64_t(nsplit)};
  cuuint64_t strides[2] = {cuuint64_t(kpad * 2), cuuint64_t(rows * kpad * 2)};
  cuuint32_t box[3] = {cuuint32_t(bk), cuuint32_t(box_rows), 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(GT_ECUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
  return GT_OK;
}

// Device error word of the tensor-core kernels (bytes 64..67 of the small
// scratch slot; bytes 0..3 hold the content-comparison flag).
int err_word(int **p) {
  void *v = nullptr;
  GT_TRY(ws_get(WS_SCRATCH4, 256, &v));
  *p = static_cast<int *>(v) + 16;
  return GT_OK;
}

template <int NSPLIT, int BK, bool CHUNKED, class Fin>
int launch_gram(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                bool symmetric, int64_t ckb, const Fin &fin, const char *prof_name,
                cudaStream_t s) {
  using C = TcCfg<NSPLIT, BK>;
  using W = SingleWork<Fin>;
  if (kpad <= 0 || kpad % BK) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  if (ckb < 1) ckb = 1;
  W w;
  GT_TRY(make_plane_map(&w.ma, zA, nA, kpad, NSPLIT, kBM, BK));
  GT_TRY(make_plane_map(&w.mb, zB, nB, kpad, NSPLIT, kBN, BK));
  w.ts = make_tiles(nA, nB, symmetric);
  w.nk = kpad / BK;
  w.fin = fin;
  if (w.ts.ntiles == 0) return GT_OK;
  int *err = nullptr;
  GT_TRY(err_word(&err));
  GT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  auto kern = gram_tc_kernel<NSPLIT, BK, CHUNKED, W>;
  GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
  const int64_t grid = w.ts.ntiles < sm_count() ? w.ts.ntiles : sm_count();
  ProfScope prof(prof_name, s);
  kern<<<unsigned(grid), kTcThreads, C::SMEM, s>>>(w, ckb, err);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

int tc_config() {
  static int cfg = -1;
  if (cfg < 0) {
    const char *e = std::getenv("GT_TC_BK");
    cfg = (e && std::atoi(e) == 32) ? 32 : 64;
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

}  // namespace

// C[r][c] = sum_k A_r[k] B_c[k] over split-bf16 planes ([part][row][kpad]),
// chunked FP32 accumulation, stored as a row-major float matrix.
int gemm_tc_store(const void *planesA, int64_t nA, const void *planesB, int64_t nB, int64_t kpad,
                  int nsplit, float *C, int64_t ldc, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  StoreFinish fin{C, ldc, nA, nB};
  if (nsplit == 3)
    return launch_gram<3, 32, true>(planesA, nA, planesB, nB, kpad, false, tc_chunk_kblocks(32),
                                    fin, "gemm_store", s);
  return launch_gram<2, 64, true>(planesA, nA, planesB, nB, kpad, false, tc_chunk_kblocks(64),
                                  fin, "gemm_store", s);
}

int tc_check_error(cudaStream_t s, bool *failed) {
  int *err = nullptr;
  GT_TRY(err_word(&err));
  int h = 0;
  GT_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  *failed = h != 0;
  if (h) GT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  return GT_OK;
}

int pearson_tc_prologue(const float *dX, int64_t nvar, int64_t n, int nsplit, int slot_z,
                        int slot_st, void **Z, int64_t *kpad, cudaStream_t s) {
  *kpad = cdiv(n, kKPad) * kKPad;
  void *pz = nullptr, *pst = nullptr;
  GT_TRY(ws_get(slot_z, size_t(nsplit) * size_t(nvar) * size_t(*kpad) * 2, &pz));
  GT_TRY(ws_get(slot_st, size_t(nvar) * sizeof(ColStats), &pst));
  ColStats *st = static_cast<ColStats *>(pst);
  ProfScope prof("pearson_prologue", s);
  GT_TRY(launch_colstats(dX, nvar, n, GT_EVERYTHING, st, s));
  auto *z = static_cast<__nv_bfloat16 *>(pz);
  if (nvar > 2147483647LL) return fail(GT_EINVAL, "too many variables");
  if (nsplit == 3)
    pearson_split_kernel<3><<<unsigned(nvar), 256, 0, s>>>(dX, nvar, n, *kpad, st, z);
  else
    pearson_split_kernel<2><<<unsigned(nvar), 256, 0, s>>>(dX, nvar, n, *kpad, st, z);
  count_launch();
  GT_CUDA(cudaGetLastError());
  *Z = pz;
  return GT_OK;
}

int pearson_tc(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad, int nsplit,
               const PearsonOut &out, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  if (!out.corr && !out.ts && !out.pairs) return GT_OK;
  PearsonFinish fin{out.corr, out.ts, out.pairs, out.ld, nA, nB, out.npairs,
                    std::sqrt(out.npairs - 2.f), out.symmetric};
  const bool sym = out.symmetric != 0;
  if (nsplit == 3)
    return launch_gram<3, 32, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(32), fin,
                                    "pearson_gram", s);
  if (tc_config() == 32)
    return launch_gram<2, 32, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(32), fin,
                                    "pearson_gram", s);
  return launch_gram<2, 64, true>(zA, nA, zB, nB, kpad, sym, tc_chunk_kblocks(64), fin,
                                  "pearson_gram", s);
}

int euclid_tc(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
              cudaStream_t st) {
  if (dim == 0 || n < 2) return dist_simt(d_pts, n, dim, d_out, layout, GT_EUCLIDEAN, 2.f, st);
  // Output writes bound this kernel at moderate dim, so the float32-level
  // 3-way split costs nothing over the 2-way one: always use it.
  constexpr int NS = 3;
  const int64_t kpad = cdiv(dim, kKPad) * kKPad;
  void *pz = nullptr, *pn = nullptr, *psum = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, size_t(NS) * size_t(n) * size_t(kpad) * 2, &pz));
  GT_TRY(ws_get(WS_SCRATCH2, size_t(n) * 4, &pn));
  GT_TRY(ws_get(WS_SCRATCH3, size_t(dim) * 8, &psum));
  auto *z = static_cast<__nv_bfloat16 *>(pz);
  auto *norm2 = static_cast<float *>(pn);
  auto *sums = static_cast<double *>(psum);
  {
    ProfScope prof("euclid_prologue", st);
    GT_CUDA(cudaMemsetAsync(sums, 0, size_t(dim) * 8, st));
    const int64_t per_block = 2048;
    dim3 cg((unsigned)cdiv(dim, 128), (unsigned)cdiv(n, per_block), 1u);
    euclid_colsum_kernel<<<cg, 128, 0, st>>>(d_pts, n, dim, per_block, sums);
    count_launch();
    int64_t g = cdiv(n * 32, 256);
    if (g > int64_t(sm_count()) * 16) g = int64_t(sm_count()) * 16;
    euclid_split_kernel<NS><<<unsigned(g), 256, 0, st>>>(d_pts, n, dim, kpad, sums, z, norm2);
    count_launch();
    GT_CUDA(cudaGetLastError());
  }
  // Entries with d^2 below an eighth of |a|^2 + |b|^2 are recomputed exactly.
  EuclidFinish fin{norm2, d_pts, d_out, n, dim, layout, 0.125f};
  return launch_gram<NS, 32, false>(z, n, z, n, kpad, true, 0, fin, "euclid_gram", st);
}

// Batched cor(x): builds device descriptors (through `alloc`, which the plan
// owns), balances the tiles over one CTA per SM, and returns the runner that
// launches prologue + Gram for the whole batch.
int pearson_batch_prepare(const gt_cor_problem *probs, int64_t count, int nsplit, int bk,
                          int64_t chunk_elems, const std::function<int(size_t, void **)> &alloc,
                          std::function<int(cudaStream_t)> *run, int64_t *ntiles_out,
                          int64_t *nctas_out) {
  std::vector<PearsonBatchInput> inputs;
  std::vector<PearsonBatchProblem> descs;
  std::vector<int64_t> var_prefix{0}, tile_prefix{0}, cost;
  int64_t plane_elems = 0, vars = 0;
  // first pass: shapes and offsets
  for (int64_t i = 0; i < count; i++) {
    const gt_cor_problem &q = probs[i];
    if (q.p < 0 || q.n < 0) return fail(GT_EINVAL, "problem %lld: negative size", (long long)i);
    if (q.p == 0) continue;
    if (!q.X) return fail(GT_EINVAL, "problem %lld: null input", (long long)i);
    if (q.n == 0) return fail(GT_EINVAL, "problem %lld: no observations", (long long)i);
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
  void *d_planes = nullptr, *d_st = nullptr, *d_in = nullptr, *d_vp = nullptr;
  GT_TRY(alloc(size_t(plane_elems) * 2, &d_planes));
  GT_TRY(alloc(size_t(vars) * sizeof(ColStats), &d_st));
  auto *planes = static_cast<__nv_bfloat16 *>(d_planes);
  int64_t ckb = chunk_elems / bk;
  if (ckb < 1) ckb = 1;
  // second pass: tensor maps, tiles, finishes
  int64_t pidx = 0;
  for (int64_t i = 0; i < count; i++) {
    const gt_cor_problem &q = probs[i];
    if (q.p == 0) continue;
    const PearsonBatchInput &b = inputs[pidx++];
    PearsonBatchProblem d;
    std::memset(&d, 0, sizeof(d));
    GT_TRY(make_plane_map(&d.map, planes + b.plane_off, b.p, b.kpad, nsplit, kBM, bk));
    d.ts = make_tiles(b.p, b.p, true);
    d.nk = b.kpad / bk;
    d.fin = PearsonFinish{q.corr, q.ts, q.pairs, b.p, b.p, b.p, float(b.n),
                          std::sqrt(float(b.n) - 2.f), 1};
    descs.push_back(d);
    tile_prefix.push_back(tile_prefix.back() + d.ts.ntiles);
    const int64_t nch = (d.nk + ckb - 1) / ckb;
    for (int64_t t = 0; t < d.ts.ntiles; t++) cost.push_back(d.nk + 2 * nch + 4);
  }
  const int64_t ntiles = tile_prefix.back();
  int64_t ncta = sm_count();
  if (ncta > ntiles) ncta = ntiles;
  std::vector<int64_t> cta_tiles, cta_off;
  if (ntiles > 0) {
    // longest-processing-time first over the CTAs
    std::vector<int64_t> order(ntiles);
    for (int64_t t = 0; t < ntiles; t++) order[t] = t;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t c) { return cost[a] > cost[c]; });
    std::vector<int64_t> load(ncta, 0);
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
      cta_tiles.insert(cta_tiles.end(), lists[c].begin(), lists[c].end());
    }
    cta_off[ncta] = int64_t(cta_tiles.size());
  }
  auto upload = [&](const void *src, size_t bytes, void **dst) -> int {
    GT_TRY(alloc(bytes, dst));
    if (bytes) GT_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return GT_OK;
  };
  void *d_desc = nullptr, *d_tp = nullptr, *d_ct = nullptr, *d_co = nullptr, *d_err = nullptr;
  GT_TRY(upload(inputs.data(), inputs.size() * sizeof(PearsonBatchInput), &d_in));
  GT_TRY(upload(var_prefix.data(), var_prefix.size() * 8, &d_vp));
  GT_TRY(upload(descs.data(), descs.size() * sizeof(PearsonBatchProblem), &d_desc));
  GT_TRY(upload(tile_prefix.data(), tile_prefix.size() * 8, &d_tp));
  GT_TRY(upload(cta_tiles.data(), cta_tiles.size() * 8, &d_ct));
  GT_TRY(upload(cta_off.data(), cta_off.size() * 8, &d_co));
  GT_TRY(alloc(256, &d_err));
  PearsonBatchWork w;
  w.probs = static_cast<const PearsonBatchProblem *>(d_desc);
  w.tile_prefix = static_cast<const int64_t *>(d_tp);
  w.nprob = nprob;
  w.cta_tiles = static_cast<const int64_t *>(d_ct);
  w.cta_off = static_cast<const int64_t *>(d_co);
  auto *in = static_cast<const PearsonBatchInput *>(d_in);
  auto *vp = static_cast<const int64_t *>(d_vp);
  auto *st = static_cast<ColStats *>(d_st);
  auto *err = static_cast<int *>(d_err);
  const int64_t total_vars = vars;
  const int ns = nsplit;
  const int BKc = bk;
  *ntiles_out = ntiles;
  *nctas_out = ncta;
  *run = [=](cudaStream_t s) -> int {
    GT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    if (total_vars == 0) return GT_OK;
    if (total_vars > 2147483647LL) return fail(GT_EINVAL, "too many variables in the batch");
    pearson_batch_stats_kernel<<<unsigned(total_vars), kColStatThreads, 0, s>>>(in, vp, nprob, st);
    if (ns == 3)
      pearson_batch_split_kernel<3><<<unsigned(total_vars), 256, 0, s>>>(in, vp, nprob, st, planes);
    else
      pearson_batch_split_kernel<2><<<unsigned(total_vars), 256, 0, s>>>(in, vp, nprob, st, planes);
    count_launch(2);
    if (ncta == 0) return GT_OK;
    if (ns == 3) {
      using C = TcCfg<3, 32>;
      auto k = gram_tc_kernel<3, 32, true, PearsonBatchWork>;
      GT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
      k<<<unsigned(ncta), kTcThreads, C::SMEM, s>>>(w, ckb, err);
    } else if (BKc == 32) {
      using C = TcCfg<2, 32>;
      auto k = gram_tc_kernel<2, 32, true, PearsonBatchWork>;
      GT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
      k<<<unsigned(ncta), kTcThreads, C::SMEM, s>>>(w, ckb, err);
    } else {
      using C = TcCfg<2, 64>;
      auto k = gram_tc_kernel<2, 64, true, PearsonBatchWork>;
      GT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
      k<<<unsigned(ncta), kTcThreads, C::SMEM, s>>>(w, ckb, err);
    }
    count_launch();
    GT_CUDA(cudaGetLastError());
    return GT_OK;
  };
  return GT_OK;
}

}  // namespace gt
