// stats.cuh -- per-variable FP64 statistics shared by the Pearson paths.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace gt {

constexpr int kColStatThreads = 256;

// Sum of v over the CTA (kColStatThreads threads), returned to every thread.
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (l < kColStatThreads / 32) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) sh[0] = t;
  }
  __syncthreads();
  return sh[0];
}

// One CTA's statistics of a variable x[0..n): FP64 mean (refined by the mean
// residual, the corrected two-pass algorithm) and centred sum of squares.
// use 0: every value counts and any NaN flags the variable; use 1: NaN values
// are skipped.  Every thread returns the same result.
__device__ __forceinline__ ColStats colstats_block(const float *__restrict__ x, int64_t n, int use,
                                                   double *sh) {
  double s = 0.0, cnt = 0.0, nan = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += kColStatThreads) {
    const float v = x[k];
    if (v != v) { nan += 1.0; continue; }
    s += double(v);
    cnt += 1.0;
  }
  s = block_sum(s, sh);
  cnt = block_sum(cnt, sh);
  nan = block_sum(nan, sh);
  double mean = cnt > 0.0 ? s / cnt : 0.0;
  double c = 0.0, ss = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += kColStatThreads) {
    const float v = x[k];
    if (v != v) continue;
    const double d = double(v) - mean;
    c += d;
    ss = fma(d, d, ss);
  }
  c = block_sum(c, sh);
  ss = block_sum(ss, sh);
  ColStats st;
  if (cnt > 0.0) {
    mean += c / cnt;
    ss -= c * c / cnt;
  }
  st.mean = mean;
  st.flags = 0;
  if (use == 0 && nan > 0.0) st.flags |= 1;
  if (!(ss > 0.0) || cnt < 2.0) st.flags |= 2;
  st.inv_norm = (st.flags & 2) ? 0.0 : 1.0 / sqrt(ss);
  return st;
}

}  // namespace gt
