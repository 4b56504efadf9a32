// stats.cuh -- per-variable statistics shared by the Pearson paths.
//
// GB300's FP64 pipe runs at a small fraction of its FP32 pipe, so the sums
// over observations are compensated float pairs (Knuth's TwoSum, squares with
// their exact FMA residual), about 2^-44 relative, and FP64 enters only in
// the few per-variable operations that finish the statistics.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.cuh"

namespace gt {

// Compensated float accumulator: hi + lo carries the sum of the added values.
struct FloatPairSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float t = hi + v;
    const float bp = t - hi;
    lo += (hi - (t - bp)) + (v - bp);
    hi = t;
  }
  __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// Sum of the lanes' (hi, lo) pairs, left in every lane.  TwoSum is exact in
// either operand order, so every lane ends with the same pair.
__device__ __forceinline__ void warp_pair_sum(float &hi, float &lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float t = hi + oh, bp = t - hi;
    lo = (lo + ol) + ((hi - (t - bp)) + (oh - bp));
    hi = t;
  }
}

// Visits x[0..n) across the warp: float4 loads when x is 16-byte aligned.
template <class F>
__device__ __forceinline__ void warp_for_each(const float *__restrict__ x, int64_t n, F &&f) {
  const int lane = threadIdx.x & 31;
  const int64_t n4 = (reinterpret_cast<uintptr_t>(x) & 15u) == 0 ? (n >> 2) : 0;
  const float4 *x4 = reinterpret_cast<const float4 *>(x);
  for (int64_t k = lane; k < n4; k += 32) {
    const float4 t = x4[k];
    f(t.x);
    f(t.y);
    f(t.z);
    f(t.w);
  }
  for (int64_t k = 4 * n4 + lane; k < n; k += 32) f(x[k]);
}

// 1/N in double from a float reciprocal and one Newton step.
__device__ __forceinline__ double recip_d(double N) {
  const double y = double(1.f / float(N));
  return y * (2.0 - N * y);
}

// Sum of x[0..n) as a float pair in every lane, with the count of non-NaN
// values, of NaN values, and the largest finite magnitude; values are
// multiplied by the power of two `sc` first.
struct WarpSums {
  double S;
  int cnt, nan;
  float amax;
};
__device__ __forceinline__ WarpSums warp_sums(const float *__restrict__ x, int64_t n, float sc) {
  const unsigned FULL = 0xffffffffu;
  FloatPairSum s;
  int cnt = 0, nan = 0;
  float amax = 0.f;
  warp_for_each(x, n, [&](float v) {
    if (v != v) {
      nan++;
    } else {
      s.add(v * sc);
      cnt++;
      const float a = fabsf(v);
      if (a <= 3.4e38f) amax = fmaxf(amax, a);
    }
  });
  float hi = s.hi, lo = s.lo;
  warp_pair_sum(hi, lo);
  WarpSums r;
  r.S = double(hi) + double(lo);
  r.cnt = __reduce_add_sync(FULL, cnt);
  r.nan = __reduce_add_sync(FULL, nan);
  r.amax = __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(amax)));
  return r;
}

// One warp's statistics of a variable x[0..n): the mean, refined by the mean
// residual (the corrected two-pass algorithm), and the inverse norm of the
// centred values.  use 0: every value counts and any NaN flags the variable;
// use 1: NaN values are skipped.  Every lane returns the same result.
// The centred pass runs on the values times 2^-e (2^e the binade of the
// largest magnitude), so its squares neither overflow nor underflow whatever
// the data's scale; the first pass is redone scaled only if its plain sum
// overflowed.  A constant variable gets a mean equal to its value (its pair
// sum is exact and the quotient is corrected), so its centred values are
// exactly 0 and it is flagged.
__device__ __forceinline__ ColStats colstats_warp(const float *__restrict__ x, int64_t n,
                                                  int use) {
  WarpSums w = warp_sums(x, n, 1.f);
  // scale 2^-e with the largest finite magnitude in [2^e, 2^(e+1))
  int e = 0;
  if (w.amax > 0.f) e = int((__float_as_uint(w.amax) >> 23) & 255u) - 127;
  e = e < -126 ? -126 : (e > 126 ? 126 : e);
  const float sc = __uint_as_float(uint32_t(127 - e) << 23);
  const double dsc = double(sc);
  double S;
  if (w.S - w.S == 0.0 || w.amax == 0.f) {
    S = w.S * dsc;
  } else {
    S = warp_sums(x, n, sc).S;  // the plain sum overflowed
  }
  const int cnt = w.cnt;
  const double N = double(cnt);
  const double invN = cnt > 0 ? recip_d(N) : 0.0;
  double mean = S * invN;                     // scaled mean
  mean = fma(fma(-mean, N, S), invN, mean);   // quotient correction
  const float mhi = float(mean), mlo = float(mean - double(mhi));
  FloatPairSum c, ss;
  float sse = 0.f;
  warp_for_each(x, n, [&](float v) {
    if (v != v) return;
    const float d = (v * sc - mhi) - mlo;
    c.add(d);
    const float q = d * d;
    sse += fmaf(d, d, -q);
    ss.add(q);
  });
  float chi = c.hi, clo = c.lo, qhi = ss.hi, qlo = ss.lo + sse;
  warp_pair_sum(chi, clo);
  warp_pair_sum(qhi, qlo);
  const double C = double(chi) + double(clo);
  double SS = double(qhi) + double(qlo);
  if (cnt > 0) {
    mean += C * invN;
    SS -= C * (C * invN);
  }
  ColStats st;
  st.mean = mean / dsc;  // exact: a power of two
  st.flags = 0;
  if (use == 0 && w.nan > 0) st.flags |= 1;
  if (!(SS > 0.0) || cnt < 2) st.flags |= 2;
  if (st.flags & 2) {
    st.inv_norm = 0.0;
  } else {
    // 1/sqrt(SS): float estimate, one Newton step in double, then the scale
    const double y = double(rsqrtf(float(SS)));
    st.inv_norm = y * (1.5 - 0.5 * SS * y * y) * dsc;
  }
  return st;
}

// z = (x - mean) * inv_norm in float arithmetic with the mean as a float
// pair: the float rounding of the FP64 value to within a couple of ulp.
struct Centerer {
  float mhi, mlo, inv;
  __device__ __forceinline__ explicit Centerer(const ColStats &s)
      : mhi(float(s.mean)), mlo(float(s.mean - double(float(s.mean)))), inv(float(s.inv_norm)) {}
  __device__ __forceinline__ float operator()(float x) const { return ((x - mhi) - mlo) * inv; }
};

}  // namespace gt
