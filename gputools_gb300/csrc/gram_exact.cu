// gram_exact.cu -- the Pearson Gram on tcgen05 tensor cores without
// accumulation error (GT_GRAM_TC_F16X6).
//
// Reference: the contraction the reference performs as one n-length float
// dot product per 16-thread block (inst/cuda/correlation.cu:248-292
// gpuPMCCNoTest, summed in float).
//
// Why.  The tensor core accumulates in FP32 and truncates each addition, so
// a Gram of floating-point split parts (f16x3, bf16x6) carries an error that
// grows with the number of additions: about 4e-7 absolute in r at 4096
// observations, which is 4e-5 relative for |r| = 0.01.  Here the operands are
// cut into fixed-point digits on one grid per variable (the error-free
// splitting of Ozaki, Ogita, Oishi and Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012), so that every product of
// digits is an integer multiple of 2^-24 and the FP32 sums of them are exact.
//
// Digits.  With z the normalised column (sum z^2 = 1, |z| <= 1), v = z * 2^11
// (so |v| <= 2^11) is held as a float pair and cut as
//   d0 = rint(v),  d1 = rint((v - d0) 2^12),  d2 = rint(((v - d0) 2^12 - d1) 2^12)
// with |d_i| <= 2^11, so P0 = d0 2^-12, X1 = d1 2^-12 and X2 = d2 2^-12 are
// exact fp16 values of magnitude <= 1/2 on the grid 2^-12 and
//   z / 2 = P0 + 2^-12 X1 + 2^-24 X2 + e,   |e| <= 2^-37.
// Then r = <z_a, z_b> = 4 (S0 + 2^-12 S1 + 2^-24 S2) up to terms below 2^-34:
//   S0 = sum P0a P0b                      |S0| <= |P0a| |P0b| ~ 1/4: exact
//   S1 = sum P0a X1b + X1a P0b            exact while |S1| < 1 (typically ~0.2)
//   S2 = sum P0a X2b + X2a P0b + X1a X1b  rounds at ~2^-44 of r
// Every term is a multiple of 2^-24, so S0 (bounded by Cauchy-Schwarz) and S1
// are exact FP32 sums, whatever the order the tensor core adds them in.  The
// three sums live in three TMEM accumulators; the epilogue forms
// r = 4 (S0 + (2^-12 S1 + 2^-24 S2)) with one rounding to float.
//
// Kernel.  Persistent, one CTA per SM, 10 warps, on the 128 x 256 tiles of
// the other Gram kernels, each processed as two 128 x 128 halves (a half that
// lies wholly below the diagonal of a symmetric problem is skipped):
//   warp 0      TMA producer: 3-D loads of the three digit planes of the A
//               (128-row) and B (128-row) boxes, 32 k per stage;
//   warp 1      allocates 512 TMEM columns (three 128 x 128 accumulators) and
//               one thread issues six tcgen05.mma (M = 128, N = 128, K = 16)
//               per k-step: P0.P0 -> S0, P0.X1, X1.P0 -> S1,
//               P0.X2, X2.P0, X1.X1 -> S2;
//   warps 2..9  epilogue: two warps per TMEM lane quarter, 64 columns each;
//               they read the three sums, release the accumulators, then run
//               the Pearson finish while the next half's MMAs run.
// Every mbarrier wait is bounded; on timeout the CTA sets the device error
// word, drains its copies and MMAs, frees TMEM and exits.
#include "common.cuh"
#include "gram_core.cuh"
#include "kernels.cuh"
#include "stats.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>

namespace gt {

namespace {

constexpr int kXB = 128;     // columns of a half tile (MMA N)
constexpr int kXBK = 32;     // k per stage (64-byte rows, 64-byte swizzle)
constexpr int kXPlanes = 3;  // digit planes P0, X1, X2
constexpr int kXEpi = 8;     // epilogue warps
constexpr int kXThreads = 64 + 32 * kXEpi;
constexpr int kXCols = 4 * kXB / kXEpi;  // columns per epilogue warp (64)
constexpr int kXATile = kBM * kXBK * 2;  // 8 KB
constexpr int kXBTile = kXB * kXBK * 2;  // 8 KB
constexpr int kXStage = kXPlanes * (kXATile + kXBTile);
constexpr int kXEpiBytes = kXEpi * kEpiTileFloats * 4;
constexpr int kXStagesRaw = (kMaxSmem - 1024 - 256 - kXEpiBytes) / kXStage;
constexpr int kXStages = kXStagesRaw > 6 ? 6 : kXStagesRaw;
constexpr int kXSmem = kXStages * kXStage + 1024 + 256 + kXEpiBytes;
static_assert(kXStages >= 3, "the exact Gram needs at least three stages");
static_assert(kXCols == 64, "two 32-column blocks per epilogue warp");

// Products of a k-step: (A plane, B plane, accumulator).
__device__ __forceinline__ void exact_product(int p, int &pa, int &pb, int &acc) {
  const int A[6] = {0, 0, 1, 0, 2, 1}, B[6] = {0, 1, 0, 2, 0, 1}, C[6] = {0, 1, 1, 2, 2, 2};
  pa = A[p];
  pb = B[p];
  acc = C[p];
}

// Whether half h of a tile holds an entry the finish writes: it starts
// inside the columns and, for a symmetric problem, reaches the diagonal.
__device__ __forceinline__ bool half_live(const PearsonFinish &fin, const TileRef &ref, int h) {
  const int64_t c0 = ref.col0 + int64_t(h) * kXB;
  if (c0 >= fin.nc) return false;
  if (fin.symmetric && c0 + kXB - 1 < ref.row0) return false;
  return true;
}

template <class Work>
__global__ void __launch_bounds__(kXThreads, 1)
gram_exact_kernel(const __grid_constant__ Work work, const tc::WaitCfg wc) {
  if (work.skip()) return;  // a gated launch whose gate is closed: before any setup
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kXStages * kXStage);
  uint64_t *empty = full + kXStages;
  uint64_t *accf = empty + kXStages;
  uint64_t *acce = accf + 1;
  uint64_t *mma_done = acce + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  float *epi_smem = reinterpret_cast<float *>(smem + kXStages * kXStage + 256);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kXStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accf, 1);
    tc::mbar_init(acce, kXEpi);
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_barrier_init();
  }
  if (warp == 0 && lane == 0) work.prefetch();
  if (warp == 1) tc::tmem_alloc(tmem_slot, 4 * kXB);
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
      bool go = true;
      while (go && !*abort_flag && tiles.next(ref)) {
        const auto &fin = work.finish(ref);
        for (int h = 0; h < 2 && go; h++) {
          if (!half_live(fin, ref, h)) continue;
          const int32_t c0 = int32_t(ref.col0 + int64_t(h) * kXB);
          for (int64_t kb = 0; kb < ref.nk; kb++, it++) {
            const int s = int(it % kXStages);
            const uint32_t use = uint32_t(it / kXStages);
            if (!tc::mbar_wait(&empty[s], (use & 1u) ^ 1u, abort_flag, wc)) {
              *abort_flag = 1;
              go = false;
              break;
            }
            uint8_t *st = smem + s * kXStage;
            tc::mbar_arrive_expect_tx(&full[s], kXStage);
#pragma unroll
            for (int p = 0; p < kXPlanes; p++)
              tc::tma_load_3d(st + p * kXATile, ref.ma, &full[s], int32_t(kb * kXBK),
                              int32_t(ref.row0), p);
#pragma unroll
            for (int p = 0; p < kXPlanes; p++)
              tc::tma_load_3d(st + kXPlanes * kXATile + p * kXBTile, ref.mb, &full[s],
                              int32_t(kb * kXBK), c0, p);
          }
        }
      }
      // drain: no bulk copy may still be writing shared memory at exit
      if (*abort_flag) {
        for (int s = 0; s < kXStages; s++) {
          const int64_t fills = it / kXStages + (s < it % kXStages ? 1 : 0);
          if (fills > 0) tc::mbar_wait_bounded(&full[s], uint32_t((fills - 1) & 1), kDrainLimitNs);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------ MMA issuer
      constexpr uint32_t idesc = tc::idesc_f32acc(kBM, kXB, 0u /* fp16 */);
      int64_t it = 0, hc = 0;
      bool ok = true;
      TileRef ref;
      TileCursor<Work> tiles(work, 0, 1);
      while (ok && tiles.next(ref)) {
        const auto &fin = work.finish(ref);
        for (int h = 0; h < 2 && ok; h++) {
          if (!half_live(fin, ref, h)) continue;
          // the epilogue has read the previous half's sums
          if (!tc::mbar_wait(acce, uint32_t(hc & 1) ^ 1u, abort_flag, wc)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          for (int64_t kb = 0; kb < ref.nk; kb++, it++) {
            const int s = int(it % kXStages);
            const uint32_t use = uint32_t(it / kXStages);
            if (!tc::mbar_wait(&full[s], use & 1u, abort_flag, wc)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(smem + s * kXStage);
            const uint32_t sb = sa + kXPlanes * kXATile;
#pragma unroll
            for (int k = 0; k < kXBK / 16; k++) {
#pragma unroll
              for (int p = 0; p < 6; p++) {
                int pa, pb, acc;
                exact_product(p, pa, pb, acc);
                const uint64_t ad = tc::smem_desc_kmajor(sa + pa * kXATile + k * 32, 64);
                const uint64_t bd = tc::smem_desc_kmajor(sb + pb * kXBTile + k * 32, 64);
                // the first product into each sum starts it
                const bool first = kb == 0 && k == 0 && (p == 0 || p == 1 || p == 3);
                tc::umma_bf16(tmem_base + uint32_t(acc * kXB), ad, bd, idesc, first ? 0u : 1u);
              }
            }
            tc::umma_commit(&empty[s]);
          }
          if (!ok) break;
          tc::umma_commit(accf);
          hc++;
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
    const int part = (warp - 2) >> 2;  // column part: 0 or 1
    EpiCtx ctx;
    ctx.wsm = epi_smem + (warp - 2) * kEpiTileFloats;
    ctx.nlist = 0;
    ctx.gcount = 0;
    int64_t hc = 0;
    bool ok = true;
    TileRef ref;
    TileCursor<Work> tiles(work, 0, 1);
    while (ok && tiles.next(ref)) {
      const auto &fin = work.finish(ref);
      for (int h = 0; h < 2; h++) {
        if (!half_live(fin, ref, h)) continue;
        const int64_t r = ref.row0 + q * 32 + lane;
        const int64_t col = ref.col0 + int64_t(h) * kXB + part * kXCols;
        ctx.rbase = r - lane;
        ctx.col0 = col;
        const bool got = tc::mbar_wait(accf, uint32_t(hc & 1), abort_flag, wc);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t tb = tmem_base + uint32_t(part * kXCols) + (uint32_t(q * 32) << 16);
        float g[2][32];
#pragma unroll
        for (int i = 0; i < 2; i++) {
          float t[32];
          tc::tmem_ld32(tb + uint32_t(2 * kXB + 32 * i), t);  // S2
#pragma unroll
          for (int j = 0; j < 32; j++) g[i][j] = t[j] * 5.9604644775390625e-8f;  // 2^-24
          tc::tmem_ld32(tb + uint32_t(kXB + 32 * i), t);  // S1
#pragma unroll
          for (int j = 0; j < 32; j++) g[i][j] = fmaf(t[j], 2.44140625e-4f, g[i][j]);  // 2^-12
          tc::tmem_ld32(tb + uint32_t(32 * i), t);  // S0
#pragma unroll
          for (int j = 0; j < 32; j++) g[i][j] += t[j];
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(acce);
        hc++;
        fin.begin_tile(r, ctx);
        fin(r, col, g[0], ctx);
        fin(r, col + 32, g[1], ctx);
        fin.end_tile(ctx);
      }
    }
    if (!ok) *abort_flag = 1;
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) atomicOr(wc.err, 1);
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_base, 4 * kXB);
  }
}

// Digits of v = vh + vl (|v| <= 2^11) as fp16 bit patterns of P0, X1, X2.
__device__ __forceinline__ void exact_digits(float vh, float vl, uint16_t (&p)[3]) {
  const float d0 = rintf(vh);
  const float wh = (vh - d0) * 4096.f;  // exact: |vh - d0| <= 1/2 on vh's grid
  const float wl = vl * 4096.f;
  const float d1 = rintf(wh + wl);
  const float e2 = (wh - d1) + wl;
  const float d2 = rintf(e2 * 4096.f);
  p[0] = __half_as_ushort(__float2half_rn(d0 * 2.44140625e-4f));
  p[1] = __half_as_ushort(__float2half_rn(d1 * 2.44140625e-4f));
  p[2] = __half_as_ushort(__float2half_rn(d2 * 2.44140625e-4f));
}

// (x - mean) * inv_norm * 2^11 as a float pair (about 2^-46 relative), from
// the FP64 statistics held as float pairs.
struct PairCenterer {
  float mhi, mlo, ihi, ilo;
  __device__ __forceinline__ explicit PairCenterer(const ColStats &s) {
    mhi = float(s.mean);
    mlo = float(s.mean - double(mhi));
    const double inv = s.inv_norm * 2048.0;
    ihi = float(inv);
    ilo = float(inv - double(ihi));
  }
  __device__ __forceinline__ void operator()(float x, float &vh, float &vl) const {
    // x - mhi exactly (TwoSum), then - mlo into the low part
    const float s = x - mhi;
    const float bp = s - x;
    const float e = (x - (s - bp)) + (-mhi - bp);
    const float l = e - mlo;
    const float ch = s + l;
    const float bq = ch - s;
    const float cl = (s - (ch - bq)) + (l - bq);
    // (ch + cl) (ihi + ilo)
    const float p = ch * ihi;
    const float pe = fmaf(ch, ihi, -p);
    const float t = fmaf(ch, ilo, fmaf(cl, ihi, pe));
    vh = p + t;
    vl = t - (vh - p);
  }
};

// Prologue: one warp per variable computes the statistics and writes the
// three digit planes ([plane][variable][kpad], zero padded); a variable with
// a NaN or without variance gets NaN digits, so every r involving it is NaN.
__global__ void __launch_bounds__(256)
pearson_exact_prep_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int64_t kpad,
                          uint16_t *__restrict__ Z) {
  const int64_t v = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (v >= nvar) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const float *x = X + v * n;
  const ColStats st = colstats_warp(x, n, GT_EVERYTHING);
  const PairCenterer cen(st);
  const bool nanrow = st.flags != 0;
  const int64_t plane = nvar * kpad;
  uint16_t *z = Z + v * kpad;
  const bool vec = (reinterpret_cast<uintptr_t>(x) & 15u) == 0 && (n & 3) == 0;
  for (int64_t k0 = 4 * int64_t(lane); k0 < kpad; k0 += 128) {
    uint32_t w[3][2] = {{0u, 0u}, {0u, 0u}, {0u, 0u}};
    if (k0 < n) {
      float xv[4];
      if (vec) {
        const float4 t = *reinterpret_cast<const float4 *>(x + k0);
        xv[0] = t.x; xv[1] = t.y; xv[2] = t.z; xv[3] = t.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; e++) xv[e] = (k0 + e < n) ? x[k0 + e] : 0.f;
      }
#pragma unroll
      for (int e = 0; e < 4; e++) {
        uint16_t p[3] = {0, 0, 0};
        if (k0 + e < n) {
          if (nanrow) {
            p[0] = p[1] = p[2] = 0x7e00;  // fp16 NaN
          } else {
            float vh, vl;
            cen(xv[e], vh, vl);
            exact_digits(vh, vl, p);
          }
        }
#pragma unroll
        for (int q = 0; q < 3; q++) w[q][e >> 1] |= uint32_t(p[q]) << (16 * (e & 1));
      }
    }
#pragma unroll
    for (int q = 0; q < 3; q++)
      *reinterpret_cast<uint2 *>(z + q * plane + k0) = make_uint2(w[q][0], w[q][1]);
  }
}

}  // namespace

int pearson_exact_prologue(const float *dX, int64_t nvar, int64_t n, int slot_z, void **Z,
                           int64_t *kpad, cudaStream_t s) {
  *kpad = cdiv(n, kKPad) * kKPad;
  void *pz = nullptr;
  GT_TRY(ws_get(slot_z, size_t(kXPlanes) * size_t(nvar) * size_t(*kpad) * 2, &pz));
  const int64_t blocks = cdiv(nvar, 8);
  if (blocks > 2147483647LL) return fail(GT_EINVAL, "too many variables");
  ProfScope prof("pearson_prologue", s);
  pearson_exact_prep_kernel<<<unsigned(blocks), 256, 0, s>>>(dX, nvar, n, *kpad,
                                                              static_cast<uint16_t *>(pz));
  count_launch();
  GT_CUDA(cudaGetLastError());
  *Z = pz;
  return GT_OK;
}

namespace {

template <class W>
int launch_exact(const W &w, int64_t ntiles, cudaStream_t s) {
  if (ntiles == 0) return GT_OK;
  tc::WaitCfg wc;
  GT_TRY(make_wait_cfg(&wc));
  auto kern = gram_exact_kernel<W>;
  GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kXSmem));
  const int64_t grid = ntiles < sm_count() ? ntiles : sm_count();
  ProfScope prof("pearson_gram", s);
  kern<<<unsigned(grid), kXThreads, kXSmem, s>>>(w, wc);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

PearsonFinish exact_finish(const PearsonOut &out, int64_t nA, int64_t nB) {
  // r = 4 (S0 + 2^-12 S1 + 2^-24 S2): the finish's scale is 4
  PearsonFinish fin{out.corr, out.ts, out.pairs, out.ld, nA, nB, out.npairs,
                    std::sqrt(out.npairs - 2.f), 4.f, out.symmetric};
  fin.gate = out.gate;
  return fin;
}

}  // namespace

int pearson_exact_band(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                       const PearsonOut &out, const int2 *tiles, int64_t ntiles, cudaStream_t s) {
  if (nA == 0 || nB == 0 || ntiles == 0) return GT_OK;
  if (kpad <= 0 || kpad % kKPad) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  using W = TableWork<PearsonFinish>;
  W w;
  GT_TRY(tc_plane_map(&w.ma, zA, nA, kpad, kXPlanes, kBM, kXBK, true));
  GT_TRY(tc_plane_map(&w.mb, zB, nB, kpad, kXPlanes, kXB, kXBK, true));
  w.tiles = tiles;
  w.ntiles = ntiles;
  w.nk = kpad / kXBK;
  w.fin = exact_finish(out, nA, nB);
  return launch_exact(w, ntiles, s);
}

int pearson_exact(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                  const PearsonOut &out, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  if (!out.corr && !out.ts && !out.pairs) return GT_OK;
  if (kpad <= 0 || kpad % kKPad) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  using W = SingleWork<PearsonFinish>;
  W w;
  GT_TRY(tc_plane_map(&w.ma, zA, nA, kpad, kXPlanes, kBM, kXBK, true));
  GT_TRY(tc_plane_map(&w.mb, zB, nB, kpad, kXPlanes, kXB, kXBK, true));
  const int mode = out.symmetric ? kUpper : kFull;
  w.ts = make_tiles(nA, nB, mode, band_group(int64_t(kBN) * kpad * 2 * kXPlanes));
  if (w.ts.ntiles > 2147483647LL)
    return fail(GT_EINVAL, "problem too large (%lld tiles)", (long long)w.ts.ntiles);
  w.nk = kpad / kXBK;
  w.fin = exact_finish(out, nA, nB);
  return launch_exact(w, w.ts.ntiles, s);
}

}  // namespace gt
