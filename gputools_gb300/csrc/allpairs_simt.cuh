// allpairs_simt.cuh -- shared-memory-tiled CUDA-core engine for all-pairs
// reductions over two row sets (distances, the FP32 Gram path of Pearson,
// pairwise-complete Pearson sums).
//
// The reference launches one 32- or 16-thread block per output entry and
// re-reads both vectors from global memory for every entry
// (inst/cuda/distance.cu:40-78 and siblings, inst/cuda/correlation.cu:7-292).
// Here a 256-thread CTA computes a BM x BN output tile: operand rows are
// staged through shared memory in BK = 16 float slabs with 128-bit coalesced
// loads (register double-buffered), and each thread keeps TM x TN
// accumulators.  Thread (ty, tx) owns rows ty + 16 i and columns tx + 16 j, so
// lanes of a warp touch consecutive output columns (coalesced stores) and the
// padded 20-float shared rows are read conflict-free.  For symmetric problems
// only tiles with ti <= tj run; off-diagonal tiles also store the mirror.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "common.cuh"

namespace gt {

constexpr int kSimtThreads = 256;
constexpr int kSimtBK = 16;
constexpr int kSimtLd = 20;  // padded shared row (floats); 80 B keeps float4 alignment

struct SimtArgs {
  const float *R;  // row operand: nr rows of K floats, stride ldr
  const float *C;  // column operand: nc rows, stride ldc
  int64_t ldr, ldc, nr, nc, K;
  int symmetric;   // R == C: only tiles ti <= tj, mirror off-diagonal tiles
  int vec_ok;      // strides and base pointers allow float4 loads
  const int *run_if = nullptr;  // when set, the kernel does nothing unless *run_if != 0
};

// Loads one BK slab of `rows` rows into registers (float4 per chunk).
template <int ROWS, class Op>
__device__ __forceinline__ void simt_load(float4 (&reg)[ROWS * 4 / kSimtThreads],
                                          const float *__restrict__ base, int64_t ld,
                                          int64_t nrows, int64_t row0, int64_t k0,
                                          int64_t K, int vec_ok) {
#pragma unroll
  for (int s = 0; s < ROWS * 4 / kSimtThreads; s++) {
    int q = threadIdx.x + s * kSimtThreads;
    int row = q >> 2, c4 = q & 3;
    int64_t gr = row0 + row, gk = k0 + c4 * 4;
    const float pad = Op::pad();
    if (gr < nrows && vec_ok && gk + 3 < K) {
      reg[s] = __ldg(reinterpret_cast<const float4 *>(base + gr * ld + gk));
    } else {
      float v[4];
#pragma unroll
      for (int e = 0; e < 4; e++)
        v[e] = (gr < nrows && gk + e < K) ? __ldg(base + gr * ld + gk + e) : pad;
      reg[s] = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
}

template <int ROWS>
__device__ __forceinline__ void simt_store(float *sm, const float4 (&reg)[ROWS * 4 / kSimtThreads]) {
#pragma unroll
  for (int s = 0; s < ROWS * 4 / kSimtThreads; s++) {
    int q = threadIdx.x + s * kSimtThreads;
    int row = q >> 2, c4 = q & 3;
    *reinterpret_cast<float4 *>(sm + row * kSimtLd + c4 * 4) = reg[s];
  }
}

// Op concept:
//   static constexpr int NACC;                 accumulators per output entry
//   static __device__ float pad();             value for rows/cols past the end
//   __device__ void init(float (&)[NACC]) const;
//   __device__ void step(float (&)[NACC], float a, float b) const;
// Out concept:
//   __device__ void operator()(int64_t r, int64_t c, const float (&acc)[NACC],
//                              bool mirror) const;
// optionally, for one value per entry whose mirror is written through shared
// memory (coalesced) instead of one scattered store per entry:
//   static constexpr bool kStagedMirror = true;
//   __device__ bool staged(bool mirror) const;       this tile goes that way
//   __device__ float value(int64_t r, int64_t c, const float (&acc)[NACC]) const;
//   __device__ void store(int64_t r, int64_t c, float v) const;
//   static constexpr bool kSkipPad = true;     optional: the last k-slab stops
//                                              at K instead of computing its padding
//                                              (for costly steps or small K; the
//                                              check slows the cheap steps down)
template <class T, class = void>
struct SkipPad : std::false_type {};
template <class T>
struct SkipPad<T, std::void_t<decltype(T::kSkipPad)>> : std::bool_constant<T::kSkipPad> {};
template <class T, class = void>
struct HasStagedMirror : std::false_type {};
template <class T>
struct HasStagedMirror<T, std::void_t<decltype(T::kStagedMirror)>>
    : std::bool_constant<T::kStagedMirror> {};
template <class Op, class Out, int TM, int TN>
__global__ void __launch_bounds__(kSimtThreads)
allpairs_simt_kernel(SimtArgs a, Op op, Out out) {
  constexpr int BM = 16 * TM, BN = 16 * TN, NA = Op::NACC;
  if (a.run_if && *a.run_if == 0) return;  // a gated launch whose gate is closed
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (a.symmetric && ti > tj) return;
  const int64_t row0 = int64_t(ti) * BM, col0 = int64_t(tj) * BN;

  __shared__ __align__(16) float sA[2][BM * kSimtLd];
  __shared__ __align__(16) float sB[2][BN * kSimtLd];

  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[TM][TN][NA];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) op.init(acc[i][j]);

  float4 ra[BM * 4 / kSimtThreads], rb[BN * 4 / kSimtThreads];
  simt_load<BM, Op>(ra, a.R, a.ldr, a.nr, row0, 0, a.K, a.vec_ok);
  simt_load<BN, Op>(rb, a.C, a.ldc, a.nc, col0, 0, a.K, a.vec_ok);
  simt_store<BM>(sA[0], ra);
  simt_store<BN>(sB[0], rb);
  __syncthreads();

  const int64_t nk = (a.K + kSimtBK - 1) / kSimtBK;
  for (int64_t kb = 0; kb < nk; kb++) {
    const int buf = int(kb & 1);
    const bool more = kb + 1 < nk;
    if (more) {
      simt_load<BM, Op>(ra, a.R, a.ldr, a.nr, row0, (kb + 1) * kSimtBK, a.K, a.vec_ok);
      simt_load<BN, Op>(rb, a.C, a.ldc, a.nc, col0, (kb + 1) * kSimtBK, a.K, a.vec_ok);
    }
    const float *pa = sA[buf];
    const float *pb = sB[buf];
#pragma unroll
    for (int kk = 0; kk < kSimtBK / 4; kk++) {
      if constexpr (SkipPad<Op>::value) {
        if (kb * kSimtBK + kk * 4 >= a.K) break;  // the last slab's padding (uniform)
      }
      float4 av[TM];
#pragma unroll
      for (int i = 0; i < TM; i++)
        av[i] = *reinterpret_cast<const float4 *>(pa + (ty + 16 * i) * kSimtLd + kk * 4);
#pragma unroll
      for (int j = 0; j < TN; j++) {
        const float4 bv = *reinterpret_cast<const float4 *>(pb + (tx + 16 * j) * kSimtLd + kk * 4);
#pragma unroll
        for (int i = 0; i < TM; i++) {
          op.step(acc[i][j], av[i].x, bv.x);
          op.step(acc[i][j], av[i].y, bv.y);
          op.step(acc[i][j], av[i].z, bv.z);
          op.step(acc[i][j], av[i].w, bv.w);
        }
      }
    }
    if (more) {
      simt_store<BM>(sA[buf ^ 1], ra);
      simt_store<BN>(sB[buf ^ 1], rb);
    }
    __syncthreads();
  }

  const bool mirror = a.symmetric && ti != tj;
  if constexpr (HasStagedMirror<Out>::value) {
    if (out.staged(mirror)) {
      // the tile's entries, then its mirror in 32-row chunks through the
      // (now idle) operand buffers: each warp writes 32 consecutive floats of
      // a mirrored row per store
      constexpr int kLdT = BN + 1;
      static_assert(32 * kLdT <= 2 * BM * kSimtLd, "a 32-row chunk fits the operand buffers");
      float *T = &sA[0][0];
#pragma unroll
      for (int i = 0; i < TM; i++) {
        const int64_t r = row0 + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < TN; j++) {
          const int64_t c = col0 + tx + 16 * j;
          const float v = out.value(r, c, acc[i][j]);
          acc[i][j][0] = v;
          if (r < a.nr && c < a.nc) out.store(r, c, v);
        }
      }
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
      for (int q = 0; q < BM / 32; q++) {
        __syncthreads();  // the previous chunk (or the main loop) is done with T
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int i = 2 * q + h;  // rows ty + 16 i of this chunk
#pragma unroll
          for (int j = 0; j < TN; j++) T[(ty + 16 * h) * kLdT + tx + 16 * j] = acc[i][j][0];
        }
        __syncthreads();
        const int64_t r = row0 + 32 * q + lane;
        for (int cc = warp; cc < BN; cc += kSimtThreads / 32) {
          const int64_t c = col0 + cc;
          if (r < a.nr && c < a.nc) out.store(c, r, T[lane * kLdT + cc]);
        }
      }
      return;
    }
  }
#pragma unroll
  for (int i = 0; i < TM; i++) {
    const int64_t r = row0 + ty + 16 * i;
    if (r >= a.nr) continue;
#pragma unroll
    for (int j = 0; j < TN; j++) {
      const int64_t c = col0 + tx + 16 * j;
      if (c >= a.nc) continue;
      out(r, c, acc[i][j], mirror);
    }
  }
}

template <class Op, class Out, int TM, int TN>
inline cudaError_t launch_allpairs_simt(const SimtArgs &a, const Op &op, const Out &out,
                                       cudaStream_t st) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  const int64_t gy = (a.nr + BM - 1) / BM, gx = (a.nc + BN - 1) / BN;
  if (gy == 0 || gx == 0) return cudaSuccess;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)gx, (unsigned)gy, 1u);
  allpairs_simt_kernel<Op, Out, TM, TN><<<grid, kSimtThreads, 0, st>>>(a, op, out);
  count_launch();
  return cudaGetLastError();
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace gt
