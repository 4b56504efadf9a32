// backward.cu -- adjoints of gpuCor (pearson) and gpuDist (euclidean), and
// the MDS stress gradient.  No counterpart in the reference (gputools has no
// differentiation); the forward quantities follow inst/cuda/correlation.cu:
// 152-292 and inst/cuda/distance.cu:40-78.
//
// Pearson.  With c_j = x_j - mean, s_j = |c_j|, z_j = c_j / s_j and
// C_ij = z_i . z_j, an upstream G = dL/dC gives
//   W = S Z  (S = G + G^T, Z the p x n matrix of the z_j),
//   dL/dx_j = (w_j - z_j (z_j . w_j)) / s_j,
// i.e. one GEMM plus a rank-1 correction per variable.  Means and norms are
// recomputed (not stored by the forward pass) with compensated float sums;
// the centring, z_j . w_j and the correction run in float arithmetic with the
// mean as a float pair and the dot product compensated (GB300's FP64 pipe is
// a small fraction of its FP32 pipe).  S and Z^T are split
// into bf16 planes and W runs on the tcgen05 chunked-accumulation kernel
// (gram_tc.cu), or on the CUDA-core engine for GT_GRAM_FP32.
//
// Distances.  dL/dx_i = sum_j W_ij (x_i - x_j) = x_i rowsum(W)_i - (W X)_i with
// W_ij = (G_ij + G_ji) / D_ij (0 where D_ij = 0), or for MDS stress
// W_ij = 2 (D_ij - delta_ij) / D_ij.  Up to 32 dimensions (64 outside 8192 ..
// 32768 points) a fused CUDA-core kernel recomputes D_ij from the points and
// never materialises W.  Otherwise the adjoint is GEMMs plus a rank-1 correction: D comes from the tcgen05
// Euclidean path (exact near-zero recomputation included), one pass over D
// and G writes W as split-bf16 planes with its row sums, W X runs on the
// tcgen05 GEMM, and dX = X diag(rowsum W) - W X is formed on the points
// centred by their column means (the gradient does not change under a
// translation, and centring keeps the two terms from cancelling).
#include "common.cuh"
#include "allpairs_simt.cuh"
#include "kernels.cuh"
#include "stats.cuh"
#include "tc_ptx.cuh"

#include <cuda_bf16.h>

namespace gt {

namespace {

constexpr int64_t kKPadB = 64;

template <class T>
__device__ __forceinline__ void put_parts(T *dst, int64_t plane, int64_t idx, float v, int ns);

template <>
__device__ __forceinline__ void put_parts<float>(float *dst, int64_t, int64_t idx, float v, int) {
  dst[idx] = v;
}

template <>
__device__ __forceinline__ void put_parts<__nv_bfloat16>(__nv_bfloat16 *dst, int64_t plane,
                                                         int64_t idx, float v, int ns) {
  uint16_t p[3];
  if (ns == 3) tc::split_parts<tc::KIND_BF16X6>(v, p);
  else tc::split_parts<tc::KIND_BF16X3>(v, p);
  for (int q = 0; q < ns; q++) dst[q * plane + idx] = __ushort_as_bfloat16(p[q]);
}

// S = G + G^T as rows j, columns i (ld kp >= p, zero padded), float or bf16
// planes.  64 x 64 tiles: the transposed operand goes through shared memory,
// loads and stores in pairs along the rows when p is even.
template <class T>
__global__ void __launch_bounds__(256)
sym_operand_kernel(const float *__restrict__ G, int64_t p, int64_t kp, int ns, T *__restrict__ S) {
  __shared__ float tile[64][65];
  const int64_t i0 = int64_t(blockIdx.x) * 64, j0 = int64_t(blockIdx.y) * 64;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool pairs = (p & 1) == 0 && (reinterpret_cast<uintptr_t>(G) & 7u) == 0;
  // tile[a][b] = G[i0 + a][j0 + b]
#pragma unroll 4
  for (int r = 0; r < 8; r++) {
    const int a = ty + 8 * r;
    const int64_t i = i0 + a, j = j0 + 2 * tx;
    float2 v = make_float2(0.f, 0.f);
    if (i < p) {
      if (pairs && j + 1 < p) {
        v = *reinterpret_cast<const float2 *>(G + i * p + j);
      } else {
        if (j < p) v.x = G[i * p + j];
        if (j + 1 < p) v.y = G[i * p + j + 1];
      }
    }
    tile[a][2 * tx] = v.x;
    tile[a][2 * tx + 1] = v.y;
  }
  __syncthreads();
  const int64_t plane = p * kp;
#pragma unroll 4
  for (int r = 0; r < 8; r++) {
    const int b = ty + 8 * r;
    const int64_t j = j0 + b, i = i0 + 2 * tx;
    if (j >= p || i >= kp) continue;
    float2 g = make_float2(0.f, 0.f);
    if (pairs && i + 1 < p) {
      g = *reinterpret_cast<const float2 *>(G + j * p + i);
    } else {
      if (i < p) g.x = G[j * p + i];
      if (i + 1 < p) g.y = G[j * p + i + 1];
    }
    const float s0 = i < p ? g.x + tile[2 * tx][b] : 0.f;
    const float s1 = i + 1 < p ? g.y + tile[2 * tx + 1][b] : 0.f;
    if constexpr (std::is_same<T, float>::value) {
      *reinterpret_cast<float2 *>(S + j * kp + i) = make_float2(s0, s1);  // kp is even
    } else {
      put_parts<T>(S, plane, j * kp + i, s0, ns);
      put_parts<T>(S, plane, j * kp + i + 1, s1, ns);
    }
  }
}

// The f16x3 operands of the Pearson adjoint without float intermediates.
// S = G + G^T is taken in 64 x 64 tile pairs: the block of (I, J), I <= J,
// loads G[I][J] and G[J][I] once and has both S[I][J] and S[J][I] = S[I][J]^T.
// Pass 1 (sym_rowmax_kernel) folds every row's largest finite |S| into
// rowmax (float bits, atomicMax); pass 2 (sym_split_kernel) scales each row
// by the power of two that brings that maximum into [2^14, 2^15) and writes
// the two f16 planes ([2][p][kp], zero padded) and the factors that undo the
// scales.  G is read twice in all, S never stored in float.
__device__ __forceinline__ void sym_pair_tiles(const float *__restrict__ G, int64_t p,
                                               float (&ta)[64][65], float (&tb)[64][65],
                                               int64_t &I0, int64_t &J0) {
  I0 = int64_t(blockIdx.y) * 64;
  J0 = int64_t(blockIdx.x) * 64;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // ta[a][b] = G[I0 + a][J0 + b], tb[a][b] = G[J0 + a][I0 + b]
#pragma unroll 4
  for (int r = 0; r < 8; r++) {
    const int a = ty + 8 * r;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int b = 2 * tx + h;
      const int64_t i = I0 + a, j = J0 + b;
      ta[a][b] = (i < p && j < p) ? G[i * p + j] : 0.f;
      const int64_t jj = J0 + a, ii = I0 + b;
      tb[a][b] = (jj < p && ii < p) ? G[jj * p + ii] : 0.f;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float finite_abs(float v) {
  const float a = fabsf(v);
  return a == a ? a : 0.f;  // NaN does not count, as fmaxf would skip it
}

__global__ void __launch_bounds__(256)
sym_rowmax_kernel(const float *__restrict__ G, int64_t p, unsigned *__restrict__ rowmax) {
  if (blockIdx.y > blockIdx.x) return;  // the pair (J, I) is done by block (I, J)
  __shared__ float ta[64][65], tb[64][65];
  __shared__ float cm[8][64];
  int64_t I0, J0;
  sym_pair_tiles(G, p, ta, tb, I0, J0);
  const int tx = threadIdx.x, ty = threadIdx.y;
  float c0 = 0.f, c1 = 0.f;  // this thread's columns b = 2 tx, 2 tx + 1 (rows J0 + b of S)
#pragma unroll 4
  for (int r = 0; r < 8; r++) {
    const int a = ty + 8 * r;
    const float s0 = finite_abs(ta[a][2 * tx] + tb[2 * tx][a]);
    const float s1 = finite_abs(ta[a][2 * tx + 1] + tb[2 * tx + 1][a]);
    c0 = fmaxf(c0, s0);
    c1 = fmaxf(c1, s1);
    // row I0 + a of S: the warp's 64 columns
    float m = fmaxf(s0, s1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (tx == 0 && I0 + a < p) atomicMax(rowmax + I0 + a, __float_as_uint(m));
  }
  cm[ty][2 * tx] = c0;
  cm[ty][2 * tx + 1] = c1;
  __syncthreads();
  const int t = ty * 32 + tx;
  if (t < 64 && J0 + t < p) {
    float m = cm[0][t];
#pragma unroll
    for (int q = 1; q < 8; q++) m = fmaxf(m, cm[q][t]);
    atomicMax(rowmax + J0 + t, __float_as_uint(m));
  }
}

__global__ void __launch_bounds__(256)
sym_split_kernel(const float *__restrict__ G, int64_t p, int64_t kp,
                 const unsigned *__restrict__ rowmax, uint16_t *__restrict__ planes,
                 float *__restrict__ scale) {
  if (blockIdx.y > blockIdx.x) return;
  __shared__ float ta[64][65], tb[64][65];
  int64_t I0, J0;
  sym_pair_tiles(G, p, ta, tb, I0, J0);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t plane = p * kp;
  // rows I0 + a, columns J0 + b (and, off the diagonal, rows J0 + a, columns I0 + b)
#pragma unroll 2
  for (int r = 0; r < 8; r++) {
    const int a = ty + 8 * r;
#pragma unroll
    for (int side = 0; side < 2; side++) {
      if (side == 1 && I0 == J0) break;
      const int64_t row = (side == 0 ? I0 : J0) + a;
      const int64_t col = (side == 0 ? J0 : I0) + 2 * tx;
      if (row >= p || col >= kp) continue;
      const int e = tc::f16_scale_exp(__uint_as_float(rowmax[row]));
      const float sc = tc::exp2i(e);
      float v[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int b = 2 * tx + h;
        // S[row][col + h]: side 0 from (a, b) of the pair, side 1 its transpose
        v[h] = side == 0 ? ta[a][b] + tb[b][a] : tb[a][b] + ta[b][a];
      }
      uint16_t h0[3], h1[3];
      tc::split_parts<tc::KIND_F16X3>(v[0] * sc, h0);
      tc::split_parts<tc::KIND_F16X3>(v[1] * sc, h1);
      *reinterpret_cast<uint32_t *>(planes + row * kp + col) = uint32_t(h0[0]) | (uint32_t(h1[0]) << 16);
      *reinterpret_cast<uint32_t *>(planes + plane + row * kp + col) =
          uint32_t(h0[1]) | (uint32_t(h1[1]) << 16);
      if (tx == 0 && side == 0 && I0 == J0) scale[row] = tc::exp2i(-e);
    }
  }
}

// Z^T as f16x3 planes ([2][n][kp], zero padded): rows k (observations),
// columns i (variables), z = (x - mean) * inv_norm.  |z| <= 1 (the centred
// variable has unit norm), so one scale, 2^14, serves every row; scale[k] =
// 2^-14 undoes it.
__global__ void __launch_bounds__(256)
zt_split_kernel(const float *__restrict__ X, int64_t p, int64_t n, int64_t kp,
                const ColStats *__restrict__ st, uint16_t *__restrict__ planes,
                float *__restrict__ scale) {
  __shared__ float tile[32][33];
  __shared__ float cen[32][4];
  const int64_t k0 = int64_t(blockIdx.x) * 32, i0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty0 = threadIdx.y;
  if (ty0 == 0) {
    const int64_t i = i0 + tx;
    if (i < p) {
      const ColStats s = st[i];
      const Centerer c(s);
      cen[tx][0] = c.mhi;
      cen[tx][1] = c.mlo;
      cen[tx][2] = c.inv;
      cen[tx][3] = s.flags ? 1.f : 0.f;
    }
    if (blockIdx.y == 0 && k0 + tx < n) scale[k0 + tx] = 1.f / 16384.f;
  }
  __syncthreads();
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t i = i0 + ty, k = k0 + tx;
    float z = 0.f;
    if (i < p && k < n && cen[ty][3] == 0.f)
      z = ((X[i * n + k] - cen[ty][0]) - cen[ty][1]) * cen[ty][2];
    tile[ty][tx] = z;  // rows i
  }
  __syncthreads();
  const int64_t plane = n * kp;
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t k = k0 + ty, i = i0 + tx;
    if (k >= n || i >= kp) continue;
    uint16_t h[3];
    tc::split_parts<tc::KIND_F16X3>(tile[tx][ty] * 16384.f, h);
    planes[k * kp + i] = h[0];
    planes[plane + k * kp + i] = h[1];
  }
}

// Z^T: rows k (observations), columns i (variables, ld kp), zero padded.
template <class T>
__global__ void zt_operand_kernel(const float *__restrict__ X, int64_t p, int64_t n, int64_t kp,
                                  const ColStats *__restrict__ st, int ns, T *__restrict__ Zt) {
  __shared__ float tile[32][33];
  __shared__ float cen[32][4];  // the block's 32 variables: mean pair, inverse norm, flag
  const int64_t k0 = int64_t(blockIdx.x) * 32, i0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty0 = threadIdx.y;
  if (ty0 == 0) {
    const int64_t i = i0 + tx;
    if (i < p) {
      const ColStats s = st[i];
      const Centerer c(s);
      cen[tx][0] = c.mhi;
      cen[tx][1] = c.mlo;
      cen[tx][2] = c.inv;
      cen[tx][3] = s.flags ? 1.f : 0.f;
    }
  }
  __syncthreads();
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t i = i0 + ty, k = k0 + tx;
    float z = 0.f;
    if (i < p && k < n && cen[ty][3] == 0.f)
      z = ((X[i * n + k] - cen[ty][0]) - cen[ty][1]) * cen[ty][2];
    tile[ty][tx] = z;  // rows i
  }
  __syncthreads();
  const int64_t plane = n * kp;
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t k = k0 + ty, i = i0 + tx;
    if (k >= n || i >= kp) continue;
    put_parts<T>(Zt, plane, k * kp + i, tile[tx][ty], ns);
  }
}

constexpr int kFinThreads = 256;

// Sum of the lanes' (hi, lo) float pairs, left in every lane (TwoSum).
__device__ __forceinline__ void warp_pair_sum_f(float &hi, float &lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float t = hi + oh, bp = t - hi;
    lo = (lo + ol) + ((hi - (t - bp)) + (oh - bp));
    hi = t;
  }
}

__device__ __forceinline__ double block_sum_d(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (l < kFinThreads / 32) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) sh[0] = t;
  }
  __syncthreads();
  return sh[0];
}

// dX_j = (w_j - z_j (z_j . w_j)) * inv_norm_j, one warp per variable: the
// dot product as a compensated float pair (each product's exact residual by
// FMA, the sums by TwoSum), the correction in float.
__global__ void __launch_bounds__(kFinThreads)
cor_backward_finish_kernel(const float *__restrict__ X, int64_t p, int64_t n,
                           const ColStats *__restrict__ st, const float *__restrict__ W,
                           float *__restrict__ dX) {
  const int64_t j = (int64_t(blockIdx.x) * kFinThreads + threadIdx.x) >> 5;
  if (j >= p) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const ColStats s = st[j];
  const float *x = X + j * n;
  const float *w = W + j * n;
  float *o = dX + j * n;
  if (s.flags) {
    for (int64_t k = lane; k < n; k += 32) o[k] = 0.f;
    return;
  }
  const Centerer cen(s);
  const float inv = float(s.inv_norm);
  float hi = 0.f, lo = 0.f;
  auto acc = [&](float xv, float wv) {
    const float z = cen(xv);
    const float pr = z * wv;
    const float pe = fmaf(z, wv, -pr);
    const float t = hi + pr, bp = t - hi;
    lo += ((hi - (t - bp)) + (pr - bp)) + pe;
    hi = t;
  };
  const bool v4 = (n & 3) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(w) |
                                    reinterpret_cast<uintptr_t>(o)) & 15u) == 0;
  if (v4) {
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    const float4 *w4 = reinterpret_cast<const float4 *>(w);
    for (int64_t k = lane; k < (n >> 2); k += 32) {
      const float4 a = x4[k], b = w4[k];
      acc(a.x, b.x);
      acc(a.y, b.y);
      acc(a.z, b.z);
      acc(a.w, b.w);
    }
  } else {
    for (int64_t k = lane; k < n; k += 32) acc(x[k], w[k]);
  }
  warp_pair_sum(hi, lo);
  const float d = hi + lo;
  if (v4) {
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    const float4 *w4 = reinterpret_cast<const float4 *>(w);
    float4 *o4 = reinterpret_cast<float4 *>(o);
    for (int64_t k = lane; k < (n >> 2); k += 32) {
      const float4 a = x4[k], b = w4[k];
      float4 r;
      r.x = fmaf(-cen(a.x), d, b.x) * inv;
      r.y = fmaf(-cen(a.y), d, b.y) * inv;
      r.z = fmaf(-cen(a.z), d, b.z) * inv;
      r.w = fmaf(-cen(a.w), d, b.w) * inv;
      o4[k] = r;
    }
  } else {
    for (int64_t k = lane; k < n; k += 32) o[k] = fmaf(-cen(x[k]), d, w[k]) * inv;
  }
}

struct OpDotB {
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const { c[0] = fmaf(a, b, c[0]); }
};

struct OutStore {
  float *out;
  int64_t ld;
  __device__ void operator()(int64_t r, int64_t c, const float (&acc)[1], bool) const {
    out[r * ld + c] = acc[0];
  }
};

// ------------------------------------------------------------ distances
constexpr int kDbRows = 128;   // rows i per CTA (one per thread)
constexpr int kDbCols = 32;    // points j per shared tile
static_assert(kDbRows / 32 == 4, "the coefficient copies step rows by four warps");

// Asynchronous 4-byte copy global -> shared (cp.async); bytes = 0 fills zero.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(tc::smem_u32(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}
// The same for 16 bytes (both addresses 16-byte aligned).
__device__ __forceinline__ void cp_async16(float *dst, const float *src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)),
               "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Shared memory of dist_backward_kernel (floats, two buffers of each tile):
// the point tile [kDbCols][DMAX], the coefficients [kDbRows][kDbCols + 1]
// (G_ij, or delta_ij from either side of the diagonal) and, for mode 0, the
// transposed coefficients [kDbCols][kDbRows + 1] (G_ji).
template <int DMAX, int MODE>
struct DbSmem {
  static constexpr int XJ = kDbCols * DMAX;
  static constexpr int CFA = kDbRows * (kDbCols + 1);
  static constexpr int CFB = MODE == 0 ? kDbCols * (kDbRows + 1) : 0;
  static constexpr int FLOATS = 2 * (XJ + CFA + CFB);  // even: the doubles after it align
  static constexpr int BYTES = FLOATS * 4 + (kDbRows / 32) * 8;
};

// mode 0: W_ij = (G_ij + G_ji) / D_ij ; mode 1: MDS, W_ij = 2 (D_ij - delta_ij) / D_ij
// CTA (ib, js): rows i of block ib against points j of split js.  Writes the
// split's partial sums sum_j W_ij x_j (pacc) and sum_j W_ij (pw), and its
// partial loss; a second kernel reduces the splits in a fixed order.
// The tiles of 32 points and their coefficients are double-buffered: the
// copies of the next tile (cp.async) run while the current one is used.
// Every thread reads the same point j at a time (a broadcast), so the point
// tile needs no padding and is read 16 bytes at a time; 1 / D_ij comes from
// the hardware reciprocal square root (D_ij = D_ij^2 / D_ij), and the stress
// sums as a compensated float pair.
template <int DMAX, int MODE>
__global__ void __launch_bounds__(kDbRows)
dist_backward_kernel(const float *__restrict__ X, int64_t n, int64_t dim,
                     const float *__restrict__ aux, int64_t jchunk, float *__restrict__ pacc,
                     float *__restrict__ pw, double *__restrict__ ploss) {
  using L = DbSmem<DMAX, MODE>;
  extern __shared__ __align__(16) float dsm[];
  float *xj = dsm;                      // [2][kDbCols][DMAX]
  float *cfa = xj + 2 * L::XJ;          // [2][kDbRows][kDbCols + 1]
  float *cfb = cfa + 2 * L::CFA;        // [2][kDbCols][kDbRows + 1] (mode 0)
  double *sh = reinterpret_cast<double *>(dsm + L::FLOATS);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t i0 = int64_t(blockIdx.x) * kDbRows;
  const int64_t i = i0 + tid;
  const int64_t js = blockIdx.y;
  const int64_t jbeg = js * jchunk;
  const int64_t jend = (jbeg + jchunk < n) ? jbeg + jchunk : n;
  // points in 16-byte copies when every row starts on a 16-byte boundary
  const bool vec = (dim & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  // copies of the tile of points jt .. jt + 31 into buffer b (one commit group);
  // the indices step from row to row (no products per copy)
  auto issue = [&](int b, int64_t jt) {
    float *xb = xj + b * L::XJ;
    if (vec) {
      for (int e = tid; e < kDbCols * DMAX / 4; e += kDbRows) {
        const int jj = e / (DMAX / 4), k = 4 * (e - jj * (DMAX / 4));
        const int64_t j = jt + jj;
        const bool ok = j < jend && k < dim;
        cp_async16(xb + 4 * e, ok ? X + j * dim + k : X, ok ? 16 : 0);
      }
    } else {
      for (int e = tid; e < kDbCols * DMAX; e += kDbRows) {
        const int jj = e / DMAX, k = e - jj * DMAX;
        const int64_t j = jt + jj;
        const bool ok = j < jend && k < dim;
        cp_async4(xb + e, ok ? X + j * dim + k : X, ok ? 4 : 0);
      }
    }
    float *ca = cfa + b * L::CFA;
    if (MODE == 0) {
      float *cb = cfb + b * L::CFB;
      const int64_t gj = jt + lane;
      int64_t gi = i0 + warp, off = gi * n + gj;  // G[gi][gj]
      for (int ii = warp; ii < kDbRows; ii += kDbRows / 32) {
        const bool ok = gi < n && gj < jend;
        cp_async4(ca + ii * (kDbCols + 1) + lane, ok ? aux + off : aux, ok ? 4 : 0);
        gi += kDbRows / 32;
        off += (kDbRows / 32) * n;
      }
      int64_t gj2 = jt, off2 = jt * n + i;  // G[gj2][i]
      for (int jj = 0; jj < kDbCols; jj++) {
        const bool ok = gj2 < jend && i < n;
        cp_async4(cb + jj * (kDbRows + 1) + tid, ok ? aux + off2 : aux, ok ? 4 : 0);
        gj2++;
        off2 += n;
      }
    } else {
      // delta in R dist layout: (a > b) at B(b) + a with B(b) = n b - b (b + 1) / 2 - b - 1;
      // each cell comes from exactly one side of the diagonal (the diagonal and
      // the cells past the tile are never read), and a side the tile does not
      // reach is skipped whole
      if (jt + kDbCols - 1 > i0) {  // cells with gj > gi: row gi, consecutive gj
        const int64_t gj = jt + lane;
        int64_t gi = i0 + warp, base = n * gi - gi * (gi + 1) / 2 - gi - 1;
        for (int ii = warp; ii < kDbRows; ii += kDbRows / 32) {
          if (gi < n && gj < jend && gj > gi)
            cp_async4(ca + ii * (kDbCols + 1) + lane, aux + (base + gj), 4);
          base += 4 * n - 4 * gi - 14;  // B(gi + 4) - B(gi)
          gi += 4;
        }
      }
      if (i0 + kDbRows - 1 > jt) {  // cells with i > gj: row gj, this thread's i
        int64_t gj = jt, base = n * gj - gj * (gj + 1) / 2 - gj - 1;
        for (int jj = 0; jj < kDbCols; jj++) {
          if (gj < jend && i < n && i > gj)
            cp_async4(ca + tid * (kDbCols + 1) + jj, aux + (base + i), 4);
          base += n - gj - 2;  // B(gj + 1) - B(gj)
          gj++;
        }
      }
    }
    cp_async_commit();
  };
  float xi[DMAX], acc[DMAX];
#pragma unroll
  for (int k = 0; k < DMAX; k++) {
    xi[k] = (i < n && k < dim) ? X[i * dim + k] : 0.f;
    acc[k] = 0.f;
  }
  float wsum = 0.f;
  FloatPairSum lsum;
  if (jbeg < jend) issue(0, jbeg);
  int b = 0;
  for (int64_t j0 = jbeg; j0 < jend; j0 += kDbCols, b ^= 1) {
    if (j0 + kDbCols < jend) {
      issue(b ^ 1, j0 + kDbCols);  // the other buffer: its last readers passed the barrier below
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // tile b complete and visible
    const float *xb = xj + b * L::XJ;
    const float *ca = cfa + b * L::CFA;
    const float *cb = cfb + b * L::CFB;
    if (i < n) {
      const int jmax = (jend - j0 < kDbCols) ? int(jend - j0) : kDbCols;
      for (int jj = 0; jj < jmax; jj++) {
        const int64_t j = j0 + jj;
        const float4 *x4 = reinterpret_cast<const float4 *>(xb + jj * DMAX);
        // four partial sums: four short dependency chains instead of one
        float q0 = 0.f, q1 = 0.f, q2 = 0.f, q3 = 0.f;
#pragma unroll
        for (int k = 0; k < DMAX / 4; k++) {
          const float4 v = x4[k];
          const float t0 = xi[4 * k] - v.x, t1 = xi[4 * k + 1] - v.y;
          const float t2 = xi[4 * k + 2] - v.z, t3 = xi[4 * k + 3] - v.w;
          q0 = fmaf(t0, t0, q0);
          q1 = fmaf(t1, t1, q1);
          q2 = fmaf(t2, t2, q2);
          q3 = fmaf(t3, t3, q3);
        }
        const float d2 = (q0 + q1) + (q2 + q3);
        if (j == i) continue;
        // 1 / d: the reciprocal square root estimate above the normal range's
        // floor, IEEE operations below it
        float inv_d = 0.f, d = 0.f;
        if (d2 >= 1e-30f) {
          inv_d = rsqrtf(d2);
          d = d2 * inv_d;
        } else if (d2 > 0.f) {
          d = sqrtf(d2);
          inv_d = 1.f / d;
        }
        const float c = MODE == 0 ? ca[tid * (kDbCols + 1) + jj] + cb[jj * (kDbRows + 1) + tid]
                                  : ca[tid * (kDbCols + 1) + jj];
        // coincident points add to the stress but not to the gradient
        if (MODE == 1 && j > i) {
          const float e = d - c;
          const float q = e * e;
          lsum.add(q);
          lsum.lo += fmaf(e, e, -q);
        }
        if (!(d2 > 0.f)) continue;
        const float w = MODE == 0 ? c * inv_d : 2.f * (d - c) * inv_d;
        wsum += w;
#pragma unroll
        for (int k = 0; k < DMAX / 4; k++) {
          const float4 v = x4[k];
          acc[4 * k] = fmaf(w, v.x, acc[4 * k]);
          acc[4 * k + 1] = fmaf(w, v.y, acc[4 * k + 1]);
          acc[4 * k + 2] = fmaf(w, v.z, acc[4 * k + 2]);
          acc[4 * k + 3] = fmaf(w, v.w, acc[4 * k + 3]);
        }
      }
    }
    __syncthreads();  // every thread is done with tile b before it is refilled
  }
  if (i < n) {
    float *pa = pacc + (js * n + i) * dim;
#pragma unroll
    for (int k = 0; k < DMAX; k++)
      if (k < dim) pa[k] = acc[k];
    pw[js * n + i] = wsum;
  }
  if (MODE == 1) {
    float lh = lsum.hi, ll = lsum.lo;
    warp_pair_sum(lh, ll);
    if (lane == 0) sh[warp] = double(lh) + double(ll);
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < kDbRows / 32; w++) t += sh[w];
      ploss[blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
  }
}

// dX_i = x_i * sum_s pw[s][i] - sum_s pacc[s][i]; splits added in order.
__global__ void dist_backward_reduce_kernel(const float *__restrict__ X, int64_t n, int64_t dim,
                                            int64_t nsplit, const float *__restrict__ pacc,
                                            const float *__restrict__ pw,
                                            float *__restrict__ dX) {
  const int64_t total = n * dim;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = e / dim;
    float w = 0.f, a = 0.f;
    for (int64_t s = 0; s < nsplit; s++) {
      w += pw[s * n + i];
      a += pacc[s * n * dim + e];
    }
    dX[e] = fmaf(X[e], w, -a);
  }
}

// The partial losses summed by one CTA in a fixed order (thread t takes
// t, t + 1024, ...; then a butterfly in each warp and across the warps), so
// the result does not depend on timing.
constexpr int kLossThreads = 1024;
__global__ void __launch_bounds__(kLossThreads)
loss_reduce_kernel(const double *__restrict__ ploss, int64_t count, double *__restrict__ loss) {
  __shared__ double sh[kLossThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < count; i += kLossThreads) t += ploss[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) sh[warp] = t;
  __syncthreads();
  if (warp == 0) {
    t = sh[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) *loss = t;
  }
}

// ---------------------------------------------- distances on the tensor cores
// Column means of the points as FP64 (compensated float sums per thread, a
// fixed-order block reduction): one CTA per dimension.
__global__ void __launch_bounds__(kFinThreads)
adj_colmean_kernel(const float *__restrict__ X, int64_t n, int64_t dim, double *__restrict__ mean) {
  __shared__ double sh[32];
  const int64_t c = blockIdx.x;
  double v = 0.0;
  float hi = 0.f, lo = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += kFinThreads) {
    const float x = X[i * dim + c];
    const float t = hi + x, bp = t - hi;
    lo += (hi - (t - bp)) + (x - bp);
    hi = t;
  }
  v = double(hi) + double(lo);
  v = block_sum_d(v, sh);
  if (threadIdx.x == 0) mean[c] = v / double(n);
}

// Centred points Xc (n x dim) and the GEMM's B operand: rows c (dimensions),
// columns j (points, ld kp, zero padded), three bf16 planes; 32 x 32 tiles
// transposed through shared memory.
__global__ void adj_points_kernel(const float *__restrict__ X, int64_t n, int64_t dim,
                                  int64_t kp, const double *__restrict__ mean,
                                  float *__restrict__ Xc, __nv_bfloat16 *__restrict__ Bt) {
  __shared__ float tile[32][33];
  const int64_t j0 = int64_t(blockIdx.x) * 32, c0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty0 = threadIdx.y;
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t j = j0 + ty, c = c0 + tx;
    float v = 0.f;
    if (j < n && c < dim) {
      v = float(double(X[j * dim + c]) - mean[c]);
      Xc[j * dim + c] = v;
    }
    tile[ty][tx] = v;  // rows j
  }
  __syncthreads();
  const int64_t plane = dim * kp;
  for (int ty = ty0; ty < 32; ty += 8) {
    const int64_t c = c0 + ty, j = j0 + tx;
    if (c >= dim || j >= kp) continue;
    put_parts<__nv_bfloat16>(Bt, plane, c * kp + j, tile[tx][ty], 3);
  }
}

// W as the GEMM's A operand (rows i, columns j, ld kp, three bf16 planes),
// from the full distance matrix D and G (MODE 0: W = (G + G^T) / D) or the
// targets delta in R's dist layout (MODE 1: W = 2 (D - delta) / D); W_ii and
// W_ij with D_ij = 0 are 0.  Per 32 x 64 tile (two columns per thread, so the
// plane stores are 4 bytes): the rows' partial sums of W (rsum[i * nbj + jb])
// and, for MODE 1, the tile's part of the stress sum_{i<j} (D - delta)^2
// (lpart[ib * nbj + jb]); both are reduced in a fixed order afterwards.  G^T,
// and delta below the diagonal (stored by column there), go through shared
// memory so that every global read is coalesced; the stress sums as
// compensated float pairs.
constexpr int kAwRows = 32, kAwCols = 64;
template <int MODE>
__global__ void __launch_bounds__(256)
adj_weight_kernel(const float *__restrict__ D, const float *__restrict__ aux, int64_t n,
                  int64_t kp, __nv_bfloat16 *__restrict__ Wp, float *__restrict__ rsum,
                  double *__restrict__ lpart) {
  // MODE 0: tt[jj][ii] = G[j][i] (64 x 32); MODE 1: tt[ii][jj] = delta(i, j), i != j (32 x 64)
  __shared__ float tt[MODE == 0 ? kAwCols : kAwRows][MODE == 0 ? kAwRows + 1 : kAwCols + 1];
  __shared__ double lsh[8];
  const int64_t i0 = int64_t(blockIdx.y) * kAwRows, j0 = int64_t(blockIdx.x) * kAwCols;
  const int tx = threadIdx.x, ty0 = threadIdx.y;
  const int64_t nbj = gridDim.x;
  if (MODE == 0) {
    for (int jj = ty0; jj < kAwCols; jj += 8) {
      const int64_t j = j0 + jj, i = i0 + tx;
      tt[jj][tx] = (j < n && i < n) ? aux[j * n + i] : 0.f;
    }
  } else {
    // above the diagonal: row i of the dist layout, consecutive j
    for (int ii = ty0; ii < kAwRows; ii += 8) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int jj = tx + 32 * h;
        const int64_t i = i0 + ii, j = j0 + jj;
        if (i < n && j < n && i < j) tt[ii][jj] = aux[n * i - i * (i + 1) / 2 + j - i - 1];
      }
    }
    // below: delta(i, j) = delta(j, i), row j of the dist layout, consecutive i
    for (int jj = ty0; jj < kAwCols; jj += 8) {
      const int64_t i = i0 + tx, j = j0 + jj;
      if (i < n && j < n && i > j) tt[tx][jj] = aux[n * j - j * (j + 1) / 2 + i - j - 1];
    }
  }
  __syncthreads();
  const int64_t plane = n * kp;
  FloatPairSum lsum;
  for (int ii = ty0; ii < kAwRows; ii += 8) {
    const int64_t i = i0 + ii;
    float w[2] = {0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int jj = 2 * tx + h;
      const int64_t j = j0 + jj;
      if (i < n && j < n && i != j) {
        const float d = D[i * n + j];
        if (MODE == 0) {
          if (d > 0.f) w[h] = __fdividef(aux[i * n + j] + tt[jj][ii], d);
        } else {
          const float del = tt[ii][jj];
          const float e = d > 0.f ? d - del : -del;  // coincident points: in the stress only
          if (d > 0.f) w[h] = __fdividef(2.f * e, d);
          if (i < j) {
            const float q = e * e;
            lsum.add(q);
            lsum.lo += fmaf(e, e, -q);
          }
        }
      }
    }
    const int64_t j = j0 + 2 * tx;  // even, and kp is a multiple of 64
    if (i < n && j < kp) {
      uint16_t a[3], b[3];
      tc::split_parts<tc::KIND_BF16X6>(w[0], a);
      tc::split_parts<tc::KIND_BF16X6>(w[1], b);
      uint32_t *dst = reinterpret_cast<uint32_t *>(Wp + i * kp + j);
#pragma unroll
      for (int q = 0; q < 3; q++)
        dst[q * (plane / 2)] = uint32_t(a[q]) | (uint32_t(b[q]) << 16);
    }
    // row sum of the tile: the 32 lanes of a row, two columns each
    float r = w[0] + w[1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (tx == 0 && i < n) rsum[i * nbj + blockIdx.x] = r;
  }
  if (MODE == 1) {
    float lh = lsum.hi, ll = lsum.lo;
    warp_pair_sum(lh, ll);
    if (tx == 0) lsh[ty0] = double(lh) + double(ll);
    __syncthreads();
    if (tx == 0 && ty0 == 0) {
      double t = 0.0;
      for (int w = 0; w < 8; w++) t += lsh[w];
      lpart[int64_t(blockIdx.y) * nbj + blockIdx.x] = t;
    }
  }
}

// dX_i = xc_i * sum_b rsum[i][b] - C_i (C = W Xc, the sum of `parts` pieces
// of n x dim), the row's partials added in order (compensated), one warp per
// point.
__global__ void adj_finish_kernel(const float *__restrict__ Xc, const float *__restrict__ C,
                                  int parts, const float *__restrict__ rsum, int64_t n,
                                  int64_t dim, int64_t nbj, float *__restrict__ dX) {
  const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  float hi = 0.f, lo = 0.f;
  for (int64_t b = lane; b < nbj; b += 32) {
    const float x = rsum[i * nbj + b];
    const float t = hi + x, bp = t - hi;
    lo += (hi - (t - bp)) + (x - bp);
    hi = t;
  }
  warp_pair_sum_f(hi, lo);
  const float r = hi + lo;
  for (int64_t c = lane; c < dim; c += 32) {
    float w = C[i * dim + c];
    for (int q = 1; q < parts; q++) w += C[int64_t(q) * n * dim + i * dim + c];
    dX[i * dim + c] = fmaf(Xc[i * dim + c], r, -w);
  }
}

template <int MODE>
int dist_backward_tc(const float *X, int64_t n, int64_t dim, const float *aux, float *dX,
                     double *loss, cudaStream_t s) {
  const int64_t kp = cdiv(n, kKPadB) * kKPadB;
  // weight tiles: rows of 32, columns of 64 covering the padded k
  const int64_t nbj = kp / kAwCols, nbi = cdiv(n, int64_t(kAwRows));
  void *pD = nullptr, *pW = nullptr, *pM = nullptr;
  // the full distance matrix (tcgen05 Gram, near-zero pairs recomputed exactly)
  GT_TRY(ws_get(WS_ADJ0, size_t(n) * size_t(n) * 4, &pD));
  float *D = static_cast<float *>(pD);
  GT_TRY(euclid_tc(X, n, dim, D, GT_LAYOUT_FULL, s));
  GT_TRY(ws_get(WS_ADJ1, size_t(3) * size_t(n) * size_t(kp) * 2, &pW));
  auto *Wp = static_cast<__nv_bfloat16 *>(pW);
  // W Xc in K pieces when its output tiles alone would leave most SMs idle
  const int64_t out_tiles = cdiv(n, int64_t(128)) * cdiv(dim, int64_t(256));
  int parts = 1;
  while (parts < 4 && out_tiles * (parts + 1) <= int64_t(sm_count())) parts++;
  // misc: means | Xc | B planes | C (parts pieces) | rsum | loss parts
  const size_t b_mean = size_t(dim) * 8, b_xc = size_t(n) * size_t(dim) * 4;
  const size_t b_bt = size_t(3) * size_t(dim) * size_t(kp) * 2, b_c = size_t(parts) * b_xc;
  const size_t b_rs = size_t(n) * size_t(nbj) * 4, b_lp = size_t(nbi) * size_t(nbj) * 8;
  auto r256 = [](size_t b) { return (b + 255) & ~size_t(255); };
  GT_TRY(ws_get(WS_ADJ2, r256(b_mean) + r256(b_xc) + r256(b_bt) + r256(b_c) + r256(b_rs) + b_lp,
                &pM));
  char *m = static_cast<char *>(pM);
  auto *mean = reinterpret_cast<double *>(m);
  auto *Xc = reinterpret_cast<float *>(m + r256(b_mean));
  auto *Bt = reinterpret_cast<__nv_bfloat16 *>(m + r256(b_mean) + r256(b_xc));
  auto *C = reinterpret_cast<float *>(m + r256(b_mean) + r256(b_xc) + r256(b_bt));
  auto *rsum = reinterpret_cast<float *>(m + r256(b_mean) + r256(b_xc) + r256(b_bt) + r256(b_c));
  auto *lp = reinterpret_cast<double *>(m + r256(b_mean) + r256(b_xc) + r256(b_bt) + r256(b_c) +
                                        r256(b_rs));
  if (nbi > 65535 || cdiv(dim, 32) > 65535) return fail(GT_EINVAL, "too many points (%lld)", (long long)n);
  const dim3 blk(32, 8);
  adj_colmean_kernel<<<unsigned(dim), kFinThreads, 0, s>>>(X, n, dim, mean);
  adj_points_kernel<<<dim3(unsigned(kp / 32), unsigned(cdiv(dim, 32))), blk, 0, s>>>(
      X, n, dim, kp, mean, Xc, Bt);
  adj_weight_kernel<MODE><<<dim3(unsigned(nbj), unsigned(nbi)), blk, 0, s>>>(
      D, aux, n, kp, Wp, rsum, lp);
  count_launch(3);
  GT_CUDA(cudaGetLastError());
  // C = W Xc on the tensor cores (rows i, columns c)
  if (parts > 1)
    GT_TRY(gemm_tc_store_ksplit(Wp, n, Bt, dim, kp, parts, &parts, C, dim, s));
  else
    GT_TRY(gemm_tc_store(Wp, n, Bt, dim, kp, 3, C, dim, s));
  adj_finish_kernel<<<unsigned(cdiv(n * 32, 256)), 256, 0, s>>>(Xc, C, parts, rsum, n, dim, nbj,
                                                                  dX);
  count_launch();
  if (MODE == 1 && loss) {
    loss_reduce_kernel<<<1, kLossThreads, 0, s>>>(lp, nbi * nbj, loss);
    count_launch();
  }
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

template <int MODE>
int launch_dist_backward(const float *X, int64_t n, int64_t dim, const float *aux, float *dX,
                         double *loss, cudaStream_t s) {
  // measured: the tensor-core form is 10-15 % faster from 33 dimensions at 8192
  // points and more (the fused kernel pads 33-64 dimensions to 64 and runs two
  // CTAs per SM there), equal at 4096 points, and up to 2.5 times slower at 32
  // dimensions and fewer.  It holds about 10 n^2 bytes of workspace, so above
  // 32768 points (11 GB) the fused kernel, which holds none, keeps those sizes.
  if (dim > 64 || (dim > 32 && n >= 8192 && n <= 32768))
    return dist_backward_tc<MODE>(X, n, dim, aux, dX, loss, s);
  const int64_t ib = cdiv(n, kDbRows);
  // the kernel for the dimension, its shared memory, and the CTAs per SM
  auto pick = [&](auto kern, int bytes) -> int {
    int per = 0;
    if (bytes > 48 * 1024)
      GT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kDbRows, bytes));
    return per;
  };
  int per_sm = 0;
  if (dim <= 16) per_sm = pick(dist_backward_kernel<16, MODE>, DbSmem<16, MODE>::BYTES);
  else if (dim <= 32) per_sm = pick(dist_backward_kernel<32, MODE>, DbSmem<32, MODE>::BYTES);
  else per_sm = pick(dist_backward_kernel<64, MODE>, DbSmem<64, MODE>::BYTES);
  if (per_sm < 1) per_sm = 1;
  // the split count whose CTAs fill whole waves best (up to four waves; more
  // splits only when they fill clearly better)
  const int64_t slots = int64_t(sm_count()) * per_sm;
  int64_t nsplit = 1;
  double best_fill = 0.0;
  for (int64_t w = 1; w <= 4; w++) {
    const int64_t ns = w * slots / ib;
    if (ns < 1) continue;
    const double fill = double(ns * ib) / double(w * slots);
    if (fill > best_fill + 0.02) {
      best_fill = fill;
      nsplit = ns;
    }
  }
  const int64_t max_split = cdiv(n, kDbCols);
  if (nsplit > max_split) nsplit = max_split;
  if (nsplit < 1) nsplit = 1;
  if (nsplit > 65535) nsplit = 65535;
  const int64_t jchunk = cdiv(cdiv(n, nsplit), kDbCols) * kDbCols;
  nsplit = cdiv(n, jchunk);
  void *pa = nullptr, *pw = nullptr, *pl = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, size_t(nsplit) * size_t(n) * size_t(dim) * 4, &pa));
  GT_TRY(ws_get(WS_SCRATCH1, size_t(nsplit) * size_t(n) * 4, &pw));
  GT_TRY(ws_get(WS_SCRATCH2, size_t(nsplit) * size_t(ib) * 8, &pl));
  const dim3 grid(unsigned(ib), unsigned(nsplit), 1u);
  float *fa = static_cast<float *>(pa), *fw = static_cast<float *>(pw);
  double *dl = static_cast<double *>(pl);
  if (dim <= 16)
    dist_backward_kernel<16, MODE><<<grid, kDbRows, DbSmem<16, MODE>::BYTES, s>>>(
        X, n, dim, aux, jchunk, fa, fw, dl);
  else if (dim <= 32)
    dist_backward_kernel<32, MODE><<<grid, kDbRows, DbSmem<32, MODE>::BYTES, s>>>(
        X, n, dim, aux, jchunk, fa, fw, dl);
  else
    dist_backward_kernel<64, MODE><<<grid, kDbRows, DbSmem<64, MODE>::BYTES, s>>>(
        X, n, dim, aux, jchunk, fa, fw, dl);
  int64_t g = cdiv(n * dim, 256);
  if (g > int64_t(sm_count()) * 8) g = int64_t(sm_count()) * 8;
  dist_backward_reduce_kernel<<<unsigned(g), 256, 0, s>>>(X, n, dim, nsplit, fa, fw, dX);
  count_launch(2);
  if (MODE == 1 && loss) {
    loss_reduce_kernel<<<1, kLossThreads, 0, s>>>(dl, ib * nsplit, loss);
    count_launch();
  }
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace

int cor_backward_impl(const float *dX, int64_t p, int64_t n, const float *dG, float *d_dX,
                      cudaStream_t s) {
  if (p == 0 || n == 0) return GT_OK;
  const int path = gt_get_gram_path();
  const int64_t kp = cdiv(p, kKPadB) * kKPadB;
  void *pst = nullptr, *pS = nullptr, *pZ = nullptr, *pW = nullptr;
  GT_TRY(ws_get(WS_SCRATCH3, size_t(p) * sizeof(ColStats), &pst));
  ColStats *st = static_cast<ColStats *>(pst);
  ProfScope prof("cor_backward", s);
  GT_TRY(launch_colstats(dX, p, n, GT_EVERYTHING, st, s));
  GT_TRY(ws_get(WS_SCRATCH4 + 0, 256, &pW));  // keep the small slot allocated
  GT_TRY(ws_get(WS_OUT2, size_t(p) * size_t(n) * 4, &pW));
  float *W = static_cast<float *>(pW);
  const dim3 blk(32, 8);
  if (path == GT_GRAM_FP32) {
    GT_TRY(ws_get(WS_SCRATCH0, size_t(p) * size_t(kp) * 4, &pS));
    GT_TRY(ws_get(WS_SCRATCH1, size_t(n) * size_t(kp) * 4, &pZ));
    sym_operand_kernel<float><<<dim3(unsigned(kp / 64), unsigned(cdiv(p, 64))), blk, 0, s>>>(
        dG, p, kp, 1, static_cast<float *>(pS));
    zt_operand_kernel<float><<<dim3(unsigned(cdiv(n, 32)), unsigned(kp / 32)), blk, 0, s>>>(
        dX, p, n, kp, st, 1, static_cast<float *>(pZ));
    count_launch(2);
    SimtArgs a;
    a.R = static_cast<float *>(pS); a.C = static_cast<float *>(pZ);
    a.ldr = a.ldc = kp;
    a.nr = p; a.nc = n; a.K = kp;
    a.symmetric = 0; a.vec_ok = 1;
    cudaError_t e = launch_allpairs_simt<OpDotB, OutStore, 8, 8>(a, OpDotB{}, OutStore{W, n}, s);
    if (e != cudaSuccess) return fail(GT_ECUDA, "adjoint GEMM launch: %s", cudaGetErrorString(e));
  } else if (path == GT_GRAM_TC_F16X3 || path == GT_GRAM_TC_F16X6) {
    // f16x3 with every operand row scaled by a power of two (G + G^T is not
    // unit-scaled; z^T is bounded by 1 and takes one scale): three products,
    // the scales undone in the store
    void *prm = nullptr, *psc = nullptr;
    GT_TRY(ws_get(WS_ADJ0, size_t(p) * 4, &prm));
    GT_TRY(ws_get(WS_ADJ2, size_t(p + n) * 4, &psc));
    GT_TRY(ws_get(WS_SCRATCH0, size_t(2) * size_t(p) * size_t(kp) * 2, &pS));
    GT_TRY(ws_get(WS_SCRATCH1, size_t(2) * size_t(n) * size_t(kp) * 2, &pZ));
    auto *rowmax = static_cast<unsigned *>(prm);
    auto *scS = static_cast<float *>(psc), *scZ = scS + p;
    GT_CUDA(cudaMemsetAsync(rowmax, 0, size_t(p) * 4, s));
    const dim3 pairs(unsigned(kp / 64), unsigned(kp / 64));
    sym_rowmax_kernel<<<pairs, blk, 0, s>>>(dG, p, rowmax);
    sym_split_kernel<<<pairs, blk, 0, s>>>(dG, p, kp, rowmax, static_cast<uint16_t *>(pS), scS);
    zt_split_kernel<<<dim3(unsigned(cdiv(n, 32)), unsigned(kp / 32)), blk, 0, s>>>(
        dX, p, n, kp, st, static_cast<uint16_t *>(pZ), scZ);
    count_launch(3);
    GT_CUDA(cudaGetLastError());
    GT_TRY(gemm_tc_store_scaled(pS, p, pZ, n, kp, scS, scZ, W, n, s));
  } else {
    const int ns = path == GT_GRAM_TC_BF16X3 ? 2 : 3;
    GT_TRY(ws_get(WS_SCRATCH0, size_t(ns) * size_t(p) * size_t(kp) * 2, &pS));
    GT_TRY(ws_get(WS_SCRATCH1, size_t(ns) * size_t(n) * size_t(kp) * 2, &pZ));
    sym_operand_kernel<__nv_bfloat16>
        <<<dim3(unsigned(kp / 64), unsigned(cdiv(p, 64))), blk, 0, s>>>(
            dG, p, kp, ns, static_cast<__nv_bfloat16 *>(pS));
    zt_operand_kernel<__nv_bfloat16><<<dim3(unsigned(cdiv(n, 32)), unsigned(kp / 32)), blk, 0, s>>>(
        dX, p, n, kp, st, ns, static_cast<__nv_bfloat16 *>(pZ));
    count_launch(2);
    GT_CUDA(cudaGetLastError());
    GT_TRY(gemm_tc_store(pS, p, pZ, n, kp, ns, W, n, s));
  }
  cor_backward_finish_kernel<<<unsigned(cdiv(p, kFinThreads / 32)), kFinThreads, 0, s>>>(
      dX, p, n, st, W, d_dX);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_cor_backward_device(const float *d_X, int64_t p, int64_t n, const float *d_G,
                                      float *d_dX, void *stream) {
  gt::clear_error();
  if (p < 0 || n < 0) return gt::fail(GT_EINVAL, "negative size");
  if (p > 2147483647LL) return gt::fail(GT_EINVAL, "too many variables");
  if (p > 0 && n > 0 && (!d_X || !d_G || !d_dX)) return gt::fail(GT_EINVAL, "null device pointer");
  return gt::cor_backward_impl(d_X, p, n, d_G, d_dX, static_cast<cudaStream_t>(stream));
}

extern "C" int gt_dist_backward_device(const float *d_X, int64_t n, int64_t dim, const float *d_G,
                                       float *d_dX, void *stream) {
  gt::clear_error();
  if (n < 0 || dim < 0) return gt::fail(GT_EINVAL, "negative size");
  if (n == 0 || dim == 0) return GT_OK;
  if (!d_X || !d_G || !d_dX) return gt::fail(GT_EINVAL, "null device pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gt::ProfScope prof("dist_backward", s);
  return gt::launch_dist_backward<0>(d_X, n, dim, d_G, d_dX, nullptr, s);
}

extern "C" int gt_mds_stress_device(const float *d_X, int64_t n, int64_t dim,
                                    const float *d_delta, float *d_dX, double *d_loss,
                                    void *stream) {
  gt::clear_error();
  if (n < 0 || dim < 0) return gt::fail(GT_EINVAL, "negative size");
  if (n == 0 || dim == 0) return GT_OK;
  if (!d_X || !d_delta || !d_dX) return gt::fail(GT_EINVAL, "null device pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gt::ProfScope prof("mds_stress", s);
  return gt::launch_dist_backward<1>(d_X, n, dim, d_delta, d_dX, d_loss, s);
}
