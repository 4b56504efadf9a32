// allpairs_simt.cuh -- shared-memory-tiled CUDA-core engine for all-pairs
// reductions over two row sets (distances, the FP32 Gram path of Pearson,
// pairwise-complete Pearson sums).
//
// The reference launches one 32- or 16-thread block per output entry and
// re-reads both vectors from global memory for every entry
// (inst/cuda/distance.cu:40-78 and siblings, inst/cuda/correlation.cu:7-292).
// Here a 256-thread CTA computes a BM x BN output tile: operand rows are
// staged through shared memory in BK = 16 float slabs with 128-bit coalesced
// loads (register double-buffered), stored k-major (one shared row per k, all
// of the slab's points side by side), and each thread keeps TM x TN
// accumulators.  Thread (ty, tx) owns the rows 64 g + 4 ty + e (g < TM / 4,
// e < 4) and the columns tx + 16 j, so lanes of a warp touch consecutive
// output columns and the stores coalesce.  The column slab is stored
// permuted so that the thread's columns 16 (4 g + e) + tx sit side by side
// too: each k step reads TM / 4 + TN / 4 conflict-free 128-bit words and
// holds only TM + TN operand values, so the 8 x 8 tiles of single-accumulator
// reductions fit 128 registers and two CTAs share an SM: one CTA's slab
// loads and output stores run under the other's arithmetic.  Every entry
// still sums its k terms in ascending order.  For symmetric problems only
// tiles with ti <= tj run; off-diagonal tiles also store the mirror.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "common.cuh"

namespace gt {

constexpr int kSimtThreads = 256;
constexpr int kSimtBK = 16;

// k-major shared slab of ROWS points: row k holds the points' values at k,
// padded by 4 floats (keeps 16-byte alignment).  The slab stores, one 4-byte
// store per k step and thread, meet two-way (row slab) or four-way (permuted
// column slab) bank conflicts; the operand reads meet none.
template <int ROWS>
constexpr int simt_ld() { return ROWS + 4; }

// The shared row of the thread's accumulator row i: 64 (i / 4) + 4 ty + i % 4.
__device__ __forceinline__ int simt_row(int i, int ty) { return 64 * (i >> 2) + 4 * ty + (i & 3); }

// Where the column slab keeps tile column c = 16 j + t: 64 (j / 4) + 4 t + j % 4.
__device__ __forceinline__ int simt_col_pos(int c) {
  const int j = c >> 4, t = c & 15;
  return 64 * (j >> 2) + 4 * t + (j & 3);
}

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

// Stores a loaded slab k-major: value k of row `row` at sm[k * LD + row], or
// for the column slab (COLS) at sm[k * LD + simt_col_pos(row)].
template <int ROWS, bool COLS>
__device__ __forceinline__ void simt_store(float *sm, const float4 (&reg)[ROWS * 4 / kSimtThreads]) {
  constexpr int LD = simt_ld<ROWS>();
#pragma unroll
  for (int s = 0; s < ROWS * 4 / kSimtThreads; s++) {
    int q = threadIdx.x + s * kSimtThreads;
    int row = q >> 2, c4 = q & 3;
    float *p = sm + (c4 * 4) * LD + (COLS ? simt_col_pos(row) : row);
    p[0] = reg[s].x;
    p[LD] = reg[s].y;
    p[2 * LD] = reg[s].z;
    p[3 * LD] = reg[s].w;
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
//   static constexpr int kUnrollK = u;         optional: unroll the slab's k loop
//                                              u times (default: fully); a fully
//                                              unrolled slab of a long step outgrows
//                                              the instruction cache
template <class T, class = void>
struct SkipPad : std::false_type {};
template <class T>
struct SkipPad<T, std::void_t<decltype(T::kSkipPad)>> : std::bool_constant<T::kSkipPad> {};
template <class T, class = void>
struct UnrollK : std::integral_constant<int, kSimtBK> {};
template <class T>
struct UnrollK<T, std::void_t<decltype(T::kUnrollK)>> : std::integral_constant<int, T::kUnrollK> {};
template <class T, class = void>
struct HasStagedMirror : std::false_type {};
template <class T>
struct HasStagedMirror<T, std::void_t<decltype(T::kStagedMirror)>>
    : std::bool_constant<T::kStagedMirror> {};
// Two CTAs per SM (at most 128 registers a thread) where the accumulators
// leave room: up to 64 of them.
template <int TM, int TN, int NACC>
constexpr int simt_min_blocks() { return TM * TN * NACC <= 64 ? 2 : 1; }

template <class Op, class Out, int TM, int TN>
__global__ void __launch_bounds__(kSimtThreads, simt_min_blocks<TM, TN, Op::NACC>())
allpairs_simt_kernel(SimtArgs a, Op op, Out out) {
  constexpr int BM = 16 * TM, BN = 16 * TN, NA = Op::NACC;
  constexpr int LDA = simt_ld<BM>(), LDB = simt_ld<BN>();
  constexpr int KU = UnrollK<Op>::value;
  static_assert(TM % 4 == 0 && TN % 4 == 0, "rows and columns are owned in groups of four");
  if (a.run_if && *a.run_if == 0) return;  // a gated launch whose gate is closed
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (a.symmetric && ti > tj) return;
  const int64_t row0 = int64_t(ti) * BM, col0 = int64_t(tj) * BN;

  __shared__ __align__(16) float sA[2][kSimtBK * LDA];
  __shared__ __align__(16) float sB[2][kSimtBK * LDB];

  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[TM][TN][NA];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) op.init(acc[i][j]);

  float4 ra[BM * 4 / kSimtThreads], rb[BN * 4 / kSimtThreads];
  simt_load<BM, Op>(ra, a.R, a.ldr, a.nr, row0, 0, a.K, a.vec_ok);
  simt_load<BN, Op>(rb, a.C, a.ldc, a.nc, col0, 0, a.K, a.vec_ok);
  simt_store<BM, false>(sA[0], ra);
  simt_store<BN, true>(sB[0], rb);
  __syncthreads();

  const int64_t nk = (a.K + kSimtBK - 1) / kSimtBK;
  for (int64_t kb = 0; kb < nk; kb++) {
    const int buf = int(kb & 1);
    const bool more = kb + 1 < nk;
    if (more) {
      simt_load<BM, Op>(ra, a.R, a.ldr, a.nr, row0, (kb + 1) * kSimtBK, a.K, a.vec_ok);
      simt_load<BN, Op>(rb, a.C, a.ldc, a.nc, col0, (kb + 1) * kSimtBK, a.K, a.vec_ok);
    }
    const float *pa = sA[buf] + 4 * ty;
    const float *pb = sB[buf] + 4 * tx;
#pragma unroll KU
    for (int kk = 0; kk < kSimtBK; kk++) {
      if constexpr (SkipPad<Op>::value) {
        if (kb * kSimtBK + kk >= a.K) break;  // the last slab's padding (uniform)
      }
      float av[TM], bv[TN];
#pragma unroll
      for (int g = 0; g < TM / 4; g++) {
        const float4 v = *reinterpret_cast<const float4 *>(pa + kk * LDA + 64 * g);
        av[4 * g] = v.x;
        av[4 * g + 1] = v.y;
        av[4 * g + 2] = v.z;
        av[4 * g + 3] = v.w;
      }
#pragma unroll
      for (int g = 0; g < TN / 4; g++) {
        const float4 v = *reinterpret_cast<const float4 *>(pb + kk * LDB + 64 * g);
        bv[4 * g] = v.x;
        bv[4 * g + 1] = v.y;
        bv[4 * g + 2] = v.z;
        bv[4 * g + 3] = v.w;
      }
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) op.step(acc[i][j], av[i], bv[j]);
    }
    if (more) {
      simt_store<BM, false>(sA[buf ^ 1], ra);
      simt_store<BN, true>(sB[buf ^ 1], rb);
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
      static_assert(32 * kLdT <= 2 * kSimtBK * LDA, "a 32-row chunk fits the operand buffers");
      float *T = &sA[0][0];
#pragma unroll
      for (int i = 0; i < TM; i++) {
        const int64_t r = row0 + simt_row(i, ty);
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
        // rows 32 q .. 32 q + 31: four rows of each thread of half the tile's ty
#pragma unroll
        for (int i = 0; i < TM; i++) {
          const int lr = simt_row(i, ty) - 32 * q;
          if (lr < 0 || lr >= 32) continue;
#pragma unroll
          for (int j = 0; j < TN; j++) T[lr * kLdT + tx + 16 * j] = acc[i][j][0];
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
    const int64_t r = row0 + simt_row(i, ty);
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
