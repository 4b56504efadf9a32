// gram_tc.cu -- split-bf16 Gram contractions on tcgen05 tensor cores, for
// Pearson (gpuCor "everything") and Euclidean distances (gpuDist).
//
// Reference: the contraction the reference performs as one n-length dot
// product per 16-thread block (inst/cuda/correlation.cu:248-292
// gpuPMCCNoTest) and as one (a-b)^2 loop per 32-thread block
// (inst/cuda/distance.cu:40-78).
//
// Operands.  Each value v (Pearson: the normalised column entry
// z = (x - mean)/||x - mean|| computed in FP64; Euclidean: the raw float
// coordinate) is split into bf16 parts v = v0 + v1 [+ v2] (round to nearest,
// each part taken from the FP64 remainder of the previous ones).  The parts
// live in separate planes [part][row][k] (K contiguous, K padded to a
// multiple of 64 with zeros).  The Gram entry is the sum of the part
// products whose order is at most NSPLIT-1:
//   NSPLIT = 2 ("bf16x3"): v0w0 + v0w1 + v1w0            (~2^-16 relative)
//   NSPLIT = 3 ("bf16x6"): + v0w2 + v1w1 + v2w0            (~2^-24: float32-exact)
// accumulated in FP32 in tensor memory.
//
// Kernel.  Persistent, one CTA per SM, 6 warps:
//   warp 0      TMA producer: 3-D tensor loads (part plane, row block, K) of
//               the A and B tiles into a STAGES-deep smem ring (128-byte or
//               64-byte swizzle), completion tracked by mbarriers;
//   warp 1      allocates 2 x BN TMEM columns (double-buffered 128 x BN FP32
//               accumulator) and one thread issues tcgen05.mma (M = 128,
//               N = BN, K = 16) for every part product, committing each stage
//               back to the producer and each finished tile to the epilogue;
//   warps 2..5  epilogue: tcgen05.ld of 32-column chunks (one TMEM lane = one
//               output row per thread) and the fused Pearson / Euclidean
//               finish, overlapped with the next tile's MMAs.
// Symmetric problems (cor(x), gpuDist) schedule only the 128 x BN tiles that
// meet the upper triangle and store each entry and its mirror.
// Every mbarrier wait is bounded: on timeout the CTA raises an error word,
// stops, releases its TMEM and exits.
#include "common.cuh"
#include "kernels.cuh"
#include "tc_ptx.cuh"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdlib>
#include <mutex>

namespace gt {

namespace {

constexpr int kTcThreads = 192;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per barrier wait
constexpr uint64_t kDrainLimitNs = 200000000ull;  // 0.2 s for in-flight work at exit
constexpr int kKPad = 64;                         // K padding of the operand planes

// ----------------------------------------------------------------- tiling
struct TileSpace {
  int64_t tr, tc;    // row blocks (128), column blocks (BN)
  int64_t j0;        // symmetric: column blocks whose tile count is 2*tj + 2
  int64_t ntiles;
  int symmetric;
};

// Symmetric problems: column block tj holds row blocks 0 .. min(2 tj + 1, tr-1)
// (the 128-row blocks that reach the upper triangle of a BN = 256 column block).
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

TileSpace make_tiles(int64_t nr, int64_t nc, int bn, bool symmetric) {
  TileSpace ts;
  ts.tr = cdiv(nr, 128);
  ts.tc = cdiv(nc, bn);
  ts.symmetric = symmetric ? 1 : 0;
  if (symmetric) {
    // requires bn == 256: column block tj meets row blocks 0 .. 2 tj + 1
    ts.j0 = ts.tr / 2;
    if (ts.j0 > ts.tc) ts.j0 = ts.tc;
    ts.ntiles = ts.j0 * (ts.j0 + 1) + (ts.tc - ts.j0) * ts.tr;
  } else {
    ts.j0 = 0;
    ts.ntiles = ts.tr * ts.tc;
  }
  return ts;
}

// ----------------------------------------------------------------- epilogues
__device__ __forceinline__ float clamp_r(float r) { return r > 1.f ? 1.f : (r < -1.f ? -1.f : r); }

__device__ __forceinline__ float signif(float r, float pairs) {
  if (r >= 0.999f) return 10000.0f;
  return r * sqrtf((pairs - 2.f) / (1.f - r * r));
}

// r = clamp(G), t-score, both orientations for cor(x).
struct PearsonEpi {
  float *corr, *ts;
  int64_t ld, nr, nc;
  float npairs;
  int symmetric;

  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32]) const {
    if (r >= nr) return;
    const bool full = c0 + 32 <= nc;
    if (full && (!symmetric || r < c0)) {
      float v[32], t[32];
#pragma unroll
      for (int j = 0; j < 32; j++) {
        v[j] = clamp_r(g[j]);
        t[j] = signif(v[j], npairs);
      }
      if (corr) {
        float4 *p = reinterpret_cast<float4 *>(corr + r * ld + c0);
        if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
          for (int j = 0; j < 8; j++) p[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
#pragma unroll
          for (int j = 0; j < 32; j++) corr[r * ld + c0 + j] = v[j];
        }
        if (symmetric)
#pragma unroll
          for (int j = 0; j < 32; j++) corr[(c0 + j) * ld + r] = v[j];
      }
      if (ts) {
        float4 *p = reinterpret_cast<float4 *>(ts + r * ld + c0);
        if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
          for (int j = 0; j < 8; j++) p[j] = make_float4(t[4 * j], t[4 * j + 1], t[4 * j + 2], t[4 * j + 3]);
        } else {
#pragma unroll
          for (int j = 0; j < 32; j++) ts[r * ld + c0 + j] = t[j];
        }
        if (symmetric)
#pragma unroll
          for (int j = 0; j < 32; j++) ts[(c0 + j) * ld + r] = t[j];
      }
      return;
    }
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const int64_t c = c0 + j;
      if (c >= nc) break;
      if (symmetric && r > c) continue;
      float v = clamp_r(g[j]);
      if (symmetric && r == c && v == v) v = 1.f;
      const float t = signif(v, npairs);
      if (corr) corr[r * ld + c] = v;
      if (ts) ts[r * ld + c] = t;
      if (symmetric && r != c) {
        if (corr) corr[c * ld + r] = v;
        if (ts) ts[c * ld + r] = t;
      }
    }
  }
};

// d^2 = |a|^2 + |b|^2 - 2 G in FP64; entries whose d^2 is below tau*(|a|^2+|b|^2),
// where the contraction's rounding could dominate, are recomputed exactly
// from the float32 points by the warp (FP64 differences), which also makes
// exact duplicates exactly 0.
struct EuclidEpi {
  const double *norm2;
  const float *pts;
  float *out;
  int64_t n, dim;
  int layout;  // GT_LAYOUT_FULL / GT_LAYOUT_DIST
  double tau;

  __device__ void operator()(int64_t r, int64_t c0, const float (&g)[32]) const {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    float v[32];
    unsigned pend = 0u;
    const double na = r < n ? norm2[r] : 0.0;
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const int64_t c = c0 + j;
      v[j] = 0.f;
      if (r < n && c < n && r < c) {
        const double nb = norm2[c];
        const double d2 = na + nb - 2.0 * double(g[j]);
        if (d2 < tau * (na + nb)) pend |= 1u << j;
        else v[j] = float(sqrt(d2));
      }
    }
    // exact recomputation of the flagged entries, one entry per warp pass
    while (true) {
      const unsigned any = __ballot_sync(FULL, pend != 0u);
      if (!any) break;
      const int src = __ffs(int(any)) - 1;
      const int j = __shfl_sync(FULL, __ffs(int(pend)) - 1, src);
      const int64_t rr = __shfl_sync(FULL, (long long)r, src);
      const int64_t c = c0 + j;
      const float *pa = pts + rr * dim, *pb = pts + c * dim;
      double acc = 0.0;
      for (int64_t k = lane; k < dim; k += 32) {
        const double d = double(pa[k]) - double(pb[k]);
        acc = fma(d, d, acc);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
      if (lane == src) {
        v[j] = float(sqrt(acc));
        pend &= ~(1u << j);
      }
    }
    if (r >= n) return;
    if (layout == GT_LAYOUT_FULL) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int64_t c = c0 + j;
        if (c >= n) break;
        if (r < c) {
          out[r * n + c] = v[j];
          out[c * n + r] = v[j];
        } else if (r == c) {
          out[r * n + c] = 0.f;
        }
      }
    } else {
      // R dist vector: entry (i = c, j = r), c > r, at n*r - r*(r+1)/2 + c - r - 1
      const int64_t base = n * r - r * (r + 1) / 2 - r - 1;
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int64_t c = c0 + j;
        if (c >= n) break;
        if (r < c) out[base + c] = v[j];
      }
    }
  }
};

// ----------------------------------------------------------------- kernel
template <int NSPLIT, int BN, int BK>
struct TcCfg {
  static constexpr int BM = 128;
  static constexpr int ROW_BYTES = BK * 2;                // 128 or 64
  static constexpr int A_TILE = BM * BK * 2;
  static constexpr int B_TILE = BN * BK * 2;
  static constexpr int STAGE = NSPLIT * (A_TILE + B_TILE);
  static constexpr int STAGES_RAW = (220 * 1024) / STAGE;
  static constexpr int STAGES = STAGES_RAW > 6 ? 6 : STAGES_RAW;
  static constexpr int SMEM = STAGES * STAGE + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr int KSTEPS = BK / 16;
  static constexpr int NPROD = NSPLIT == 2 ? 3 : 6;
  static_assert(STAGES >= 2, "need at least two stages");
  static_assert(2 * BN <= 512, "accumulators exceed TMEM");
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

template <int NSPLIT, int BN, int BK, class Epi>
__global__ void __launch_bounds__(kTcThreads, 1)
gram_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
               TileSpace tiles, int64_t nk, Epi epi, int *err) {
  using C = TcCfg<NSPLIT, BN, BK>;
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

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      tc::mbar_init(&accf[b], 1);
      tc::mbar_init(&acce[b], 4);
    }
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_barrier_init();
  }
  if (warp == 0 && lane == 0) {
    tc::prefetch_tensormap(&mapA);
    tc::prefetch_tensormap(&mapB);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, 2 * BN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------ TMA producer
      int64_t it = 0;
      for (int64_t t = blockIdx.x; t < tiles.ntiles && !*abort_flag; t += gridDim.x) {
        int64_t ti, tj;
        tile_coords(tiles, t, ti, tj);
        for (int64_t kb = 0; kb < nk; kb++, it++) {
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
            tc::tma_load_3d(st + p * C::A_TILE, &mapA, &full[s], int32_t(kb * BK),
                            int32_t(ti * C::BM), p);
#pragma unroll
          for (int p = 0; p < NSPLIT; p++)
            tc::tma_load_3d(st + NSPLIT * C::A_TILE + p * C::B_TILE, &mapB, &full[s],
                            int32_t(kb * BK), int32_t(tj * BN), p);
        }
      }
      // drain: wait (bounded) for loads that were issued but not consumed, so
      // no bulk copy is still writing shared memory when the CTA exits
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
      constexpr uint32_t idesc = tc::idesc_bf16_f32(128, BN);
      int64_t it = 0, local = 0;
      for (int64_t t = blockIdx.x; t < tiles.ntiles; t += gridDim.x, local++) {
        const int buf = int(local & 1);
        const uint32_t ause = uint32_t(local >> 1);
        if (!tc::mbar_wait(&acce[buf], (ause & 1u) ^ 1u, abort_flag, kWaitLimitNs)) {
          *abort_flag = 1;
          break;
        }
        tc::tc_fence_after();
        const uint32_t d = tmem_base + uint32_t(buf * BN);
        bool ok = true;
        for (int64_t kb = 0; kb < nk; kb++, it++) {
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
              tc::umma_bf16(d, ad, bd, idesc, (kb | k | p) != 0 ? 1u : 0u);
            }
          }
          tc::umma_commit(&empty[s]);
        }
        if (!ok) {
          *abort_flag = 1;
          break;
        }
        tc::umma_commit(&accf[buf]);
      }
      // every MMA issued above has finished before TMEM is released
      tc::umma_commit(mma_done);
      tc::mbar_wait_bounded(mma_done, 0u, kDrainLimitNs);
    }
    __syncwarp();
  } else {
    // -------------------------------------------------- epilogue (warps 2..5)
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    int64_t local = 0;
    for (int64_t t = blockIdx.x; t < tiles.ntiles; t += gridDim.x, local++) {
      int64_t ti, tj;
      tile_coords(tiles, t, ti, tj);
      const int buf = int(local & 1);
      const uint32_t ause = uint32_t(local >> 1);
      const bool ok = tc::mbar_wait(&accf[buf], ause & 1u, abort_flag, kWaitLimitNs);
      if (!__all_sync(0xffffffffu, ok)) {
        *abort_flag = 1;
        break;
      }
      tc::tc_fence_after();
      const int64_t r = ti * 128 + q * 32 + lane;
      const uint32_t tbase = tmem_base + uint32_t(buf * BN) + (uint32_t(q * 32) << 16);
#pragma unroll 1
      for (int c = 0; c < BN; c += 32) {
        float g[32];
        tc::tmem_ld32(tbase + uint32_t(c), g);
        epi(r, tj * BN + c, g);
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acce[buf]);
    }
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) atomicExch(err, 1);
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem_base, 2 * BN);
  }
}

// ----------------------------------------------------------------- operands
// Split of one FP64 value into bf16 parts (round to nearest each time).
template <int NSPLIT>
__device__ __forceinline__ void split_bf16(double z, __nv_bfloat16 (&p)[3]) {
  double rem = z;
#pragma unroll
  for (int i = 0; i < NSPLIT; i++) {
    p[i] = __double2bfloat16(rem);
    rem -= double(__bfloat162float(p[i]));
  }
}

// Pearson operand planes: z = (x - mean) * inv_norm, NaN rows for variables
// that are NaN-flagged or constant; k >= n is zero.
template <int NSPLIT>
__global__ void pearson_split_kernel(const float *__restrict__ X, int64_t nvar, int64_t n,
                                     int64_t kpad, const ColStats *__restrict__ st,
                                     __nv_bfloat16 *__restrict__ Z) {
  const int64_t total = nvar * kpad;
  const int64_t plane = total;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t v = i / kpad, k = i - v * kpad;
    __nv_bfloat16 p[3];
    if (k >= n) {
      p[0] = p[1] = p[2] = __float2bfloat16(0.f);
    } else {
      const ColStats s = st[v];
      if (s.flags) {
        p[0] = p[1] = p[2] = __float2bfloat16(__int_as_float(0x7fc00000));
      } else {
        split_bf16<NSPLIT>((double(X[v * n + k]) - s.mean) * s.inv_norm, p);
      }
    }
#pragma unroll
    for (int q = 0; q < NSPLIT; q++) Z[q * plane + i] = p[q];
  }
}

// Euclidean operand planes (raw coordinates) and FP64 squared norms, one warp
// per point.
template <int NSPLIT>
__global__ void euclid_split_kernel(const float *__restrict__ P, int64_t n, int64_t dim,
                                    int64_t kpad, __nv_bfloat16 *__restrict__ Z,
                                    double *__restrict__ norm2) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int64_t plane = n * kpad;
  for (int64_t v = warp; v < n; v += nwarps) {
    double acc = 0.0;
    for (int64_t k = lane; k < kpad; k += 32) {
      __nv_bfloat16 p[3];
      if (k < dim) {
        const double x = P[v * dim + k];
        acc = fma(x, x, acc);
        split_bf16<NSPLIT>(x, p);
      } else {
        p[0] = p[1] = p[2] = __float2bfloat16(0.f);
      }
#pragma unroll
      for (int q = 0; q < NSPLIT; q++) Z[q * plane + v * kpad + k] = p[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) norm2[v] = acc;
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

// 3-D map over planes [NSPLIT][rows][kpad] of bf16; box {BK, box_rows, 1}.
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

template <int NSPLIT, int BN, int BK, class Epi>
int launch_gram(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                bool symmetric, const Epi &epi, const char *prof_name, cudaStream_t s) {
  using C = TcCfg<NSPLIT, BN, BK>;
  if (symmetric && BN != 256) return fail(GT_EINVAL, "symmetric tiling needs BN = 256");
  if (kpad <= 0 || kpad % BK) return fail(GT_EINVAL, "bad padded K (%lld)", (long long)kpad);
  CUtensorMap mA, mB;
  GT_TRY(make_plane_map(&mA, zA, nA, kpad, NSPLIT, 128, BK));
  GT_TRY(make_plane_map(&mB, zB, nB, kpad, NSPLIT, BN, BK));
  const TileSpace ts = make_tiles(nA, nB, BN, symmetric);
  if (ts.ntiles == 0) return GT_OK;
  int *err = nullptr;
  GT_TRY(err_word(&err));
  GT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  auto kern = gram_tc_kernel<NSPLIT, BN, BK, Epi>;
  GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
  const int64_t grid = ts.ntiles < sm_count() ? ts.ntiles : sm_count();
  ProfScope prof(prof_name, s);
  kern<<<unsigned(grid), kTcThreads, C::SMEM, s>>>(mA, mB, ts, kpad / BK, epi, err);
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

__global__ void fill_kernel(float *__restrict__ p, int64_t count, float v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count;
       i += int64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

}  // namespace

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
  const int64_t total = nvar * *kpad;
  int64_t g = cdiv(total, 256);
  if (g > int64_t(sm_count()) * 16) g = int64_t(sm_count()) * 16;
  if (g < 1) g = 1;
  auto *z = static_cast<__nv_bfloat16 *>(pz);
  if (nsplit == 3)
    pearson_split_kernel<3><<<unsigned(g), 256, 0, s>>>(dX, nvar, n, *kpad, st, z);
  else
    pearson_split_kernel<2><<<unsigned(g), 256, 0, s>>>(dX, nvar, n, *kpad, st, z);
  count_launch();
  GT_CUDA(cudaGetLastError());
  *Z = pz;
  return GT_OK;
}

int pearson_tc(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad, int nsplit,
               const PearsonOut &out, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  PearsonEpi epi{out.corr, out.ts, out.ld, nA, nB, out.npairs, out.symmetric};
  if (out.pairs) {
    const int64_t count = nA * nB;
    int64_t g = cdiv(count, 256);
    if (g > int64_t(sm_count()) * 16) g = int64_t(sm_count()) * 16;
    fill_kernel<<<unsigned(g), 256, 0, s>>>(out.pairs, count, out.npairs);
    count_launch();
  }
  if (!out.corr && !out.ts) return GT_OK;
  const bool sym = out.symmetric != 0;
  if (nsplit == 3) {
    if (sym || tc_config() == 32)
      return launch_gram<3, 256, 32>(zA, nA, zB, nB, kpad, sym, epi, "pearson_gram", s);
    return launch_gram<3, 128, 64>(zA, nA, zB, nB, kpad, sym, epi, "pearson_gram", s);
  }
  if (tc_config() == 32)
    return launch_gram<2, 256, 32>(zA, nA, zB, nB, kpad, sym, epi, "pearson_gram", s);
  return launch_gram<2, 256, 64>(zA, nA, zB, nB, kpad, sym, epi, "pearson_gram", s);
}

int euclid_tc(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
              cudaStream_t st) {
  if (dim == 0 || n < 2) return dist_simt(d_pts, n, dim, d_out, layout, GT_EUCLIDEAN, 2.f, st);
  const int nsplit = gt_get_gram_path() == GT_GRAM_TC_BF16X3 ? 2 : 3;
  const int64_t kpad = cdiv(dim, kKPad) * kKPad;
  void *pz = nullptr, *pn = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, size_t(nsplit) * size_t(n) * size_t(kpad) * 2, &pz));
  GT_TRY(ws_get(WS_SCRATCH2, size_t(n) * 8, &pn));
  auto *z = static_cast<__nv_bfloat16 *>(pz);
  auto *norm2 = static_cast<double *>(pn);
  {
    ProfScope prof("euclid_prologue", st);
    int64_t g = cdiv(n * 32, 256);
    if (g > int64_t(sm_count()) * 16) g = int64_t(sm_count()) * 16;
    if (nsplit == 3)
      euclid_split_kernel<3><<<unsigned(g), 256, 0, st>>>(d_pts, n, dim, kpad, z, norm2);
    else
      euclid_split_kernel<2><<<unsigned(g), 256, 0, st>>>(d_pts, n, dim, kpad, z, norm2);
    count_launch();
    GT_CUDA(cudaGetLastError());
  }
  // Recompute entries whose d^2 is below this fraction of |a|^2 + |b|^2.
  const double tau = nsplit == 3 ? 1.0 / 64.0 : 1.0 / 4.0;
  EuclidEpi epi{norm2, d_pts, d_out, n, dim, layout, tau};
  if (nsplit == 3) return launch_gram<3, 256, 32>(z, n, z, n, kpad, true, epi, "euclid_gram", st);
  if (tc_config() == 32) return launch_gram<2, 256, 32>(z, n, z, n, kpad, true, epi, "euclid_gram", st);
  return launch_gram<2, 256, 64>(z, n, z, n, kpad, true, epi, "euclid_gram", st);
}

}  // namespace gt
