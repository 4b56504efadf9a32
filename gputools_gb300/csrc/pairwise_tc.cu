// pairwise_tc.cu -- gpuCor(method = "pearson", use = "pairwise.complete.obs")
// on tcgen05 tensor cores, for inputs with missing values.
//
// Reference: the pairwise-complete branch of the correlation kernels
// (inst/cuda/correlation.cu:7-150, driven by src/correlation.cpp:125-134):
// per pair of variables, the observations where both are present give the
// count, the two sums, the two sums of squares and the cross sum, and r
// follows from them.
//
// Here the six sums of every pair are Gram contractions over observations:
// with m_i the presence mask of variable i, z_i its values standardised by
// its own mean and norm (0 where missing) and q_i = z_i^2,
//   N = <m_i, m_j>, Sa = <z_i, m_j>, Sb = <m_i, z_j>, Saa = <q_i, m_j>,
//   Sbb = <m_i, q_j>, Sab = <z_i, z_j>.
// Five fp16 planes per variable hold m (exact), z and q as two fp16 parts
// each (times 2^14, as the f16x3 encoding: |z| <= 1).  A tile pairs 128 row
// variables (TMEM lanes) with 32 column variables whose five planes are
// stacked into one 160-row B operand [m; z hi; z lo; q hi; q lo], so each
// k-step issues six MMAs into three TMEM regions and every sum of a pair sits
// in the lane of its row variable:
//   R1 (160 columns)  A = m      x B rows 0..159: N, Sb hi, Sb lo, Sbb hi, Sbb lo
//   R2 ( 64 columns)  A = z hi   x B rows 0..63 : Sa, Sab (hi.hi)
//                     A = z lo   x B rows 0..63 : Sa, Sab (lo.hi)   (accumulated)
//                     A = z hi   x B rows 64..95: Sab (hi.lo), into R2's Sab columns
//   R4 ( 32 columns)  A = q hi, q lo x B rows 0..31: Saa
// 256 columns in all, so TMEM holds two accumulator sets and the MMAs of one
// chunk run while the epilogue reads the other.  K is accumulated in chunks of
// 256 observations (the tensor core's FP32 accumulation truncates every add);
// the epilogue adds each chunk into FP32 running sums and forms r, the t-score
// and the pair count from them.
//
// Kernel layout as in gram_tc.cu: persistent, one CTA per SM; warp 0 issues
// the TMA loads, warp 1 the MMAs, warps 2..17 are the epilogue (4 per TMEM
// lane quarter, 8 column variables each).  Every mbarrier wait is bounded.
#include "common.cuh"
#include "kernels.cuh"
#include "stats.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>

#include <vector>

namespace gt {

namespace {

constexpr int kPM = 128;                           // row variables per tile
constexpr int kPN = 32;                            // column variables per tile
constexpr int kPBK = 32;                           // observations per k-block
constexpr int kPlanes = 5;                         // m, z hi, z lo, q hi, q lo
constexpr int kPChunkKb = 8;                       // k-blocks per chunk: 256 observations
constexpr int kPStages = 4;
constexpr int kPA = kPM * kPBK * 2;                // one A plane box: 8 KB
constexpr int kPB = kPN * kPBK * 2;                // one B plane box: 2 KB
constexpr int kPStage = kPlanes * (kPA + kPB);     // 50 KB
constexpr int kPEpi = 16;                          // epilogue warps
constexpr int kPThreads = 64 + 32 * kPEpi;         // + producer and MMA warps
constexpr int kPSmem = kPStages * kPStage + 1024 + 256;
constexpr int kR1 = 0, kR2 = 160, kR4 = 224;  // TMEM columns of the regions
constexpr int kPAcc = 256;                      // columns of one accumulator set (two fit)
constexpr uint64_t kPDrainNs = 200000000ull;
constexpr float kPScale = 16384.f;                 // 2^14

struct PairwiseArgs {
  CUtensorMap ma, mb;  // 3-D maps over the five planes; boxes of 128 and 32 rows
  const int2 *tiles;   // (first row variable, first column variable) per tile
  int64_t ntiles, nk;  // tiles, k-blocks
  float *corr, *ts, *pairs;
  int64_t ld, nr, nc;
  int symmetric;
  const int *run_if;   // when set, the kernel does nothing unless *run_if != 0
};

// The five planes of one variable x[0..n): one warp, statistics over the
// present values (a variable with fewer than two, or with zero variance,
// gets z = 0 and so NaN for every r).
__global__ void __launch_bounds__(256)
pairwise_prep_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int64_t kpad,
                     uint16_t *__restrict__ P, const int *run_if) {
  if (run_if && *run_if == 0) return;
  const int64_t v = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (v >= nvar) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const float *x = X + v * n;
  const ColStats st = colstats_warp(x, n, 1);
  const Centerer cen(st);
  const bool flat = (st.flags & 2) != 0;
  const int64_t plane = nvar * kpad;
  uint16_t *p = P + v * kpad;
  for (int64_t k0 = 4 * int64_t(lane); k0 < kpad; k0 += 128) {
    uint32_t w[kPlanes][2] = {};
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int64_t k = k0 + e;
      const float val = k < n ? x[k] : __int_as_float(0x7fc00000);
      const bool present = val == val;
      const float z = (present && !flat) ? cen(val) : 0.f;
      const float zs = z * kPScale, qs = z * z * kPScale;
      const __half zh = __float2half_rn(zs), qh = __float2half_rn(qs);
      const __half zl = __float2half_rn(zs - __half2float(zh));
      const __half ql = __float2half_rn(qs - __half2float(qh));
      const uint16_t parts[kPlanes] = {present ? uint16_t(0x3c00) : uint16_t(0),
                                       __half_as_ushort(zh), __half_as_ushort(zl),
                                       __half_as_ushort(qh), __half_as_ushort(ql)};
#pragma unroll
      for (int q = 0; q < kPlanes; q++) w[q][e >> 1] |= uint32_t(parts[q]) << (16 * (e & 1));
    }
#pragma unroll
    for (int q = 0; q < kPlanes; q++)
      *reinterpret_cast<uint2 *>(p + q * plane + k0) = make_uint2(w[q][0], w[q][1]);
  }
}

// Two 8-column TMEM loads and their wait in one statement, so that no use
// of the registers can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld8x2(uint32_t a0, uint32_t a1, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%16];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%17];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(a0), "r"(a1)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float signif_pw(float r, float pairs) {
  if (r >= 0.999f) return 10000.0f;
  return r * sqrtf((pairs - 2.f) / (1.f - r * r));
}

__global__ void __launch_bounds__(kPThreads, 1)
pairwise_tc_kernel(const __grid_constant__ PairwiseArgs a, const tc::WaitCfg wc) {
  if (a.run_if && *a.run_if == 0) return;  // a gated launch whose gate is closed
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kPStages * kPStage);
  uint64_t *empty = full + kPStages;
  uint64_t *accf = empty + kPStages;
  uint64_t *acce = accf + 2;
  uint64_t *mma_done = acce + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kPStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      tc::mbar_init(&accf[b], 1);
      tc::mbar_init(&acce[b], kPEpi);
    }
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_barrier_init();
  }
  if (warp == 0 && lane == 0) {
    tc::prefetch_tensormap(&a.ma);
    tc::prefetch_tensormap(&a.mb);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int64_t nch = (a.nk + kPChunkKb - 1) / kPChunkKb;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------ TMA producer
      int64_t it = 0;
      for (int64_t t = blockIdx.x; t < a.ntiles && !*abort_flag; t += gridDim.x) {
        const int2 tl = a.tiles[t];
        for (int64_t kb = 0; kb < a.nk; kb++, it++) {
          const int s = int(it % kPStages);
          const uint32_t use = uint32_t(it / kPStages);
          if (!tc::mbar_wait(&empty[s], (use & 1u) ^ 1u, abort_flag, wc)) {
            *abort_flag = 1;
            break;
          }
          uint8_t *st = smem + s * kPStage;
          tc::mbar_arrive_expect_tx(&full[s], kPStage);
#pragma unroll
          for (int p = 0; p < kPlanes; p++)
            tc::tma_load_3d(st + p * kPA, &a.ma, &full[s], int32_t(kb * kPBK), tl.x, p);
#pragma unroll
          for (int p = 0; p < kPlanes; p++)
            tc::tma_load_3d(st + kPlanes * kPA + p * kPB, &a.mb, &full[s], int32_t(kb * kPBK),
                            tl.y, p);
        }
      }
      if (*abort_flag) {
        for (int s = 0; s < kPStages; s++) {
          const int64_t fills = it / kPStages + (s < it % kPStages ? 1 : 0);
          if (fills > 0) tc::mbar_wait_bounded(&full[s], uint32_t((fills - 1) & 1), kPDrainNs);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------ MMA issuer
      constexpr uint32_t id160 = tc::idesc_f32acc(kPM, 160, 0);
      constexpr uint32_t id64 = tc::idesc_f32acc(kPM, 64, 0);
      constexpr uint32_t id32 = tc::idesc_f32acc(kPM, 32, 0);
      int64_t it = 0, cc = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
        for (int64_t ch = 0; ch < nch && ok; ch++, cc++) {
          // two accumulator sets: wait until the epilogue has read the set's
          // previous chunk
          const int buf = int(cc & 1);
          if (!tc::mbar_wait(&acce[buf], uint32_t((cc >> 1) & 1) ^ 1u, abort_flag, wc)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t d = tmem_base + uint32_t(buf * kPAcc);
          const int64_t kb0 = ch * kPChunkKb;
          const int64_t kb1 = kb0 + kPChunkKb < a.nk ? kb0 + kPChunkKb : a.nk;
          for (int64_t kb = kb0; kb < kb1; kb++, it++) {
            const int s = int(it % kPStages);
            const uint32_t use = uint32_t(it / kPStages);
            if (!tc::mbar_wait(&full[s], use & 1u, abort_flag, wc)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(smem + s * kPStage);
            const uint32_t sb = sa + kPlanes * kPA;
#pragma unroll
            for (int k = 0; k < kPBK / 16; k++) {
              const uint32_t acc = (kb != kb0 || k) ? 1u : 0u;
              const uint64_t am = tc::smem_desc_kmajor(sa + 0 * kPA + k * 32, 64);
              const uint64_t azh = tc::smem_desc_kmajor(sa + 1 * kPA + k * 32, 64);
              const uint64_t azl = tc::smem_desc_kmajor(sa + 2 * kPA + k * 32, 64);
              const uint64_t aqh = tc::smem_desc_kmajor(sa + 3 * kPA + k * 32, 64);
              const uint64_t aql = tc::smem_desc_kmajor(sa + 4 * kPA + k * 32, 64);
              const uint64_t b0 = tc::smem_desc_kmajor(sb + k * 32, 64);            // rows 0..
              const uint64_t b2 = tc::smem_desc_kmajor(sb + 2 * kPB + k * 32, 64);  // rows 64..
              tc::umma_bf16(d + kR1, am, b0, id160, acc);
              tc::umma_bf16(d + kR2, azh, b0, id64, acc);
              tc::umma_bf16(d + kR2, azl, b0, id64, 1u);
              tc::umma_bf16(d + kR2 + 32, azh, b2, id32, 1u);  // after the two above
              tc::umma_bf16(d + kR4, aqh, b0, id32, acc);
              tc::umma_bf16(d + kR4, aql, b0, id32, 1u);
            }
            tc::umma_commit(&empty[s]);
          }
          if (ok) tc::umma_commit(&accf[buf]);
        }
      }
      if (!ok) *abort_flag = 1;
      tc::umma_commit(mma_done);
      tc::mbar_wait_bounded(mma_done, 0u, kPDrainNs);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ epilogue (warps 2..17)
    const int q = warp & 3;            // TMEM lane quarter
    const int part = (warp - 2) >> 2;  // 8 column variables: part * 8 ..
    const uint32_t lanes = uint32_t(q * 32) << 16;
    int64_t cc = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
      const int2 tl = a.tiles[t];
      float sN[8], sA[8], sB[8], sAA[8], sBB[8], sAB[8];
#pragma unroll
      for (int j = 0; j < 8; j++) sN[j] = sA[j] = sB[j] = sAA[j] = sBB[j] = sAB[j] = 0.f;
      for (int64_t ch = 0; ch < nch; ch++, cc++) {
        const int buf = int(cc & 1);
        const bool got = tc::mbar_wait(&accf[buf], uint32_t((cc >> 1) & 1), abort_flag, wc);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t tb = tmem_base + lanes + uint32_t(buf * kPAcc + part * 8);
        float v[16];
        tmem_ld8x2(tb + kR1, tb + kR1 + 32, v);  // N, Sb hi
#pragma unroll
        for (int j = 0; j < 8; j++) {
          sN[j] += v[j];
          sB[j] += v[8 + j];
        }
        tmem_ld8x2(tb + kR1 + 64, tb + kR1 + 96, v);  // Sb lo, Sbb hi
#pragma unroll
        for (int j = 0; j < 8; j++) {
          sB[j] += v[j];
          sBB[j] += v[8 + j];
        }
        tmem_ld8x2(tb + kR1 + 128, tb + kR2, v);  // Sbb lo, Sa
#pragma unroll
        for (int j = 0; j < 8; j++) {
          sBB[j] += v[j];
          sA[j] += v[8 + j];
        }
        tmem_ld8x2(tb + kR2 + 32, tb + kR4, v);  // Sab (hi.hi + lo.hi + hi.lo), Saa
#pragma unroll
        for (int j = 0; j < 8; j++) {
          sAB[j] += v[j];
          sAA[j] += v[8 + j];
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&acce[buf]);
      }
      if (!ok) break;
      const int64_t r = int64_t(tl.x) + q * 32 + lane;
      const float inv = 1.f / kPScale;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int64_t c = int64_t(tl.y) + part * 8 + j;
        if (r >= a.nr || c >= a.nc) continue;
        if (a.symmetric && r > c) continue;  // the mirror of a computed entry
        // float from the float sums (the FP64 form gains nothing once they
        // are rounded, and its registers would spill)
        const float N = sN[j];
        float val = __int_as_float(0x7fc00000);
        if (N >= 2.f) {
          const float sa = sA[j] * inv, sb = sB[j] * inv;
          const float invN = 1.f / N;
          const float va = fmaf(-sa, sa * invN, sAA[j] * inv);
          const float vb = fmaf(-sb, sb * invN, sBB[j] * inv);
          const float cv = fmaf(-sa, sb * invN, sAB[j] * (inv * inv));
          if (va > 0.f && vb > 0.f) {
            const float rr = cv / sqrtf(va * vb);
            val = rr > 1.f ? 1.f : (rr < -1.f ? -1.f : rr);
          }
        }
        if (a.symmetric && r == c && val == val) val = 1.f;
        const float np = N;
        const float tsv = signif_pw(val, np);
        const int64_t i0 = r * a.ld + c, i1 = c * a.ld + r;
        const bool mirror = a.symmetric && r != c;
        // streaming stores: the outputs, written once, leave the operand
        // planes in L2
        if (a.corr) {
          tc::st_stream(a.corr + i0, val);
          if (mirror) tc::st_stream(a.corr + i1, val);
        }
        if (a.ts) {
          tc::st_stream(a.ts + i0, tsv);
          if (mirror) tc::st_stream(a.ts + i1, tsv);
        }
        if (a.pairs) {
          tc::st_stream(a.pairs + i0, np);
          if (mirror) tc::st_stream(a.pairs + i1, np);
        }
      }
    }
    if (!ok) *abort_flag = 1;
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) atomicOr(wc.err, 1);
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_base, 512);
  }
}

}  // namespace

// Pairwise-complete Pearson of A (nA variables) against B (nB; B == A when
// symmetric) on the tensor cores, for inputs with missing values; run_if (a
// device flag, may be null) gates every launch.
int pearson_pairwise_tc(const float *dA, int64_t nA, const float *dB, int64_t nB, int64_t n,
                        const PearsonOut &out, const int *run_if, cudaStream_t s) {
  if (nA == 0 || nB == 0 || n == 0) return GT_OK;
  if (nA > 2147483647LL - kPM || nB > 2147483647LL - kPN)
    return fail(GT_EINVAL, "too many variables");
  const bool sym = out.symmetric != 0;
  const int64_t kpad = cdiv(n, 64) * 64;
  const size_t bytesA = size_t(kPlanes) * size_t(nA) * size_t(kpad) * 2;
  const size_t bytesB = sym ? 0 : size_t(kPlanes) * size_t(nB) * size_t(kpad) * 2;
  // tiles: 128 row variables x 32 column variables; for cor(x) those that
  // reach the upper triangle (column block tj >= 4 ti)
  const int64_t tr = cdiv(nA, kPM), tcn = cdiv(nB, kPN);
  std::vector<int2> tiles;
  for (int64_t ti = 0; ti < tr; ti++)
    for (int64_t tj = sym ? 4 * ti : 0; tj < tcn; tj++)
      tiles.push_back(make_int2(int(ti * kPM), int(tj * kPN)));
  if (tiles.empty()) return GT_OK;
  const size_t tbytes = tiles.size() * sizeof(int2);
  void *pw = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, bytesA + bytesB + tbytes, &pw));
  auto *pa = static_cast<uint16_t *>(pw);
  auto *pb = sym ? pa : pa + bytesA / 2;
  auto *dtiles = reinterpret_cast<int2 *>(static_cast<char *>(pw) + bytesA + bytesB);
  GT_CUDA(cudaMemcpyAsync(dtiles, tiles.data(), tbytes, cudaMemcpyHostToDevice, s));
  {
    ProfScope prof("pearson_prologue", s);
    pairwise_prep_kernel<<<unsigned(cdiv(nA, 8)), 256, 0, s>>>(dA, nA, n, kpad, pa, run_if);
    count_launch();
    if (!sym) {
      pairwise_prep_kernel<<<unsigned(cdiv(nB, 8)), 256, 0, s>>>(dB, nB, n, kpad, pb, run_if);
      count_launch();
    }
    GT_CUDA(cudaGetLastError());
  }
  PairwiseArgs a{};
  GT_TRY(tc_plane_map(&a.ma, pa, nA, kpad, kPlanes, kPM, kPBK, true));
  GT_TRY(tc_plane_map(&a.mb, pb, nB, kpad, kPlanes, kPN, kPBK, true));
  a.tiles = dtiles;
  a.ntiles = int64_t(tiles.size());
  a.nk = kpad / kPBK;
  a.corr = out.corr;
  a.ts = out.ts;
  a.pairs = out.pairs;
  a.ld = out.ld;
  a.nr = nA;
  a.nc = nB;
  a.symmetric = sym ? 1 : 0;
  a.run_if = run_if;
  tc::WaitCfg wc;
  GT_TRY(device_error_word(&wc.err));
  wc.limit_ns = wait_limit_ns();
  wc.hint_ns = wait_sleep_hint_ns();
  GT_CUDA(cudaFuncSetAttribute(pairwise_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kPSmem));
  const int64_t grid = a.ntiles < sm_count() ? a.ntiles : sm_count();
  ProfScope prof("pearson_pairwise", s);
  pairwise_tc_kernel<<<unsigned(grid), kPThreads, kPSmem, s>>>(a, wc);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace gt
