// mi.cu -- gpuMi: B-spline mutual information of every pair of variables.
//
// Reference: R/gpuMi.R -> rBSplineMutualInfo (src/rinterface.cpp:415-422) ->
// bSplineMutualInfo (src/mi.cpp:33-164), whose kernels (inst/cuda/mi.cu)
// scale each variable to [0, knot_max], give each sample its B-spline weights
// over the bins (Cox-de Boor), take the entropy of each variable and, per
// pair and per pair of bins, the joint probability as a sum over samples.
//
// Here one warp per variable scales it, computes its weights and entropy,
// and writes the weights as f16x3 planes (rows = variable x 2^lg bins, zero
// padded; weights <= 1 times 2^14); the joint probabilities of all pairs are
// then the blocks of one Gram matrix of those rows, on tcgen05 tensor cores,
// whose epilogue reduces each pair's block to sum p log2 p and adds the
// entropies (gram_tc.cu, MiFinish).  More than 32 bins, or the FP32 Gram
// path, take a CUDA-core kernel (one CTA per pair).
#include "common.cuh"
#include "kernels.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>

namespace gt {

namespace {

constexpr int kMiMaxOrder = 8;
constexpr int kMiMaxTcBins = 32;

// initKnots (src/mi.cpp:14-30) in closed form: order zeros, 1, 2, ..., then
// nbins - order + 1 repeated.
__device__ __forceinline__ float mi_knot(int i, int nbins, int order) {
  const int v = i - order + 1;
  return float(v < 0 ? 0 : (v > nbins - order + 1 ? nbins - order + 1 : v));
}

// do_fraction (inst/cuda/mi.cu:27-36)
__device__ __forceinline__ float mi_frac(float numer, float denom) {
  if (numer == denom && numer != 0.f) return 1.f;
  if (denom != 0.f) return numer / denom;
  return 0.f;
}

// The ORDER weights b[0..ORDER) of bins base .. base + ORDER - 1 for the
// scaled sample z, by the recursion and index bounds of get_bin_scores
// (inst/cuda/mi.cu:39-86), in float as there.
template <int ORDER>
__device__ __forceinline__ void mi_weights(float z, int nbins, int &base, float (&b)[ORDER + 1]) {
  const int nknots = nbins + ORDER;
  int i0 = int(floorf(z)) + ORDER - 1;
  if (i0 >= nbins) i0 = nbins - 1;
  base = i0 - ORDER + 1;
#pragma unroll
  for (int u = 0; u <= ORDER; u++) b[u] = u == ORDER - 1 ? 1.f : 0.f;
#pragma unroll
  for (int i = 2; i <= ORDER; i++) {
#pragma unroll
    for (int jj = 0; jj < i; jj++) {
      const int j = i0 - i + 1 + jj;
      const int u = ORDER - i + jj;  // j - base
      float t1 = 0.f, t2 = 0.f;
      if (!(j < 0 || j >= nbins || j >= nknots || j + i - 1 < 0 || j > nknots))
        t1 = mi_frac(z - mi_knot(j, nbins, ORDER),
                     mi_knot(j + i - 1, nbins, ORDER) - mi_knot(j, nbins, ORDER)) * b[u];
      if (!(j + 1 < 0 || j + 1 >= nbins || j + 1 >= nknots || j + i < 0 || j + i >= nknots))
        t2 = mi_frac(mi_knot(j + i, nbins, ORDER) - z,
                     mi_knot(j + i, nbins, ORDER) - mi_knot(j + 1, nbins, ORDER)) * b[u + 1];
      b[u] = t1 + t2;
    }
  }
}

// Per variable (one warp): the scale (scale(), inst/cuda/mi.cu:3-25; a
// variable with max == min, which the reference divides by zero, is taken as
// all zeros), the weights and the entropy (get_entropy, inst/cuda/mi.cu:88-113).
// planes: f16x3 rows v * 2^lg + a (TC path); wts: float [v][a][k] (CUDA-core
// path).  One of the two is null.
template <int ORDER>
__global__ void __launch_bounds__(256)
mi_prep_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int nbins, int lg,
               int64_t kpad, uint16_t *__restrict__ planes, float *__restrict__ wts,
               float *__restrict__ entropy) {
  const unsigned FULL = 0xffffffffu;
  const int64_t v = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (v >= nvar) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const float *x = X + v * n;
  float mn = x[0], mx = x[0];
  for (int64_t k = lane; k < n; k += 32) {
    mn = fminf(mn, x[k]);
    mx = fmaxf(mx, x[k]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(FULL, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
  }
  const float kmax = float(nbins - ORDER + 1);
  const float delta = mx - mn;
  const int nbp = 1 << lg;
  const int64_t rows = nvar * int64_t(nbp), plane = rows * kpad;
  float acc[kMiMaxTcBins];
#pragma unroll
  for (int a = 0; a < kMiMaxTcBins; a++) acc[a] = 0.f;
  const int64_t kend = planes ? kpad : n;
  for (int64_t k = lane; k < kend; k += 32) {
    int base = 0;
    float b[ORDER + 1];
    const bool real = k < n;
    if (real) {
      const float z = delta > 0.f ? (kmax * (x[k] - mn)) / delta : 0.f;
      mi_weights<ORDER>(z, nbins, base, b);
    }
    if (planes) {
#pragma unroll
      for (int a = 0; a < kMiMaxTcBins; a++) {
        if (a >= nbp) break;
        float w = 0.f;
#pragma unroll
        for (int u = 0; u < ORDER; u++)
          if (real && a == base + u) w = b[u];
        acc[a] += w;
        const float ws = w * 16384.f;
        const __half h = __float2half_rn(ws);
        const __half l = __float2half_rn(ws - __half2float(h));
        const int64_t row = v * nbp + a;
        planes[row * kpad + k] = __half_as_ushort(h);
        planes[plane + row * kpad + k] = __half_as_ushort(l);
      }
    } else {
      for (int a = 0; a < nbins; a++) {
        float w = 0.f;
#pragma unroll
        for (int u = 0; u < ORDER; u++)
          if (a == base + u) w = b[u];
        wts[(v * nbins + a) * n + k] = w;
      }
    }
  }
  if (planes) {
    float h = 0.f;
#pragma unroll
    for (int a = 0; a < kMiMaxTcBins; a++) {
      if (a >= nbp) break;
      float s = acc[a];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
      const float p = s / float(n);
      if (p > 0.f) h -= p * log2f(p);
    }
    if (lane == 0) entropy[v] = h;
  }
}

// Entropies of the CUDA-core layout, one warp per variable.
__global__ void __launch_bounds__(256)
mi_entropy_kernel(const float *__restrict__ wts, int64_t nvar, int64_t n, int nbins,
                  float *__restrict__ entropy) {
  const unsigned FULL = 0xffffffffu;
  const int64_t v = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (v >= nvar) return;
  const int lane = threadIdx.x & 31;
  float h = 0.f;
  for (int a = 0; a < nbins; a++) {
    const float *w = wts + (v * nbins + a) * n;
    float s = 0.f;
    for (int64_t k = lane; k < n; k += 32) s += w[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    const float p = s / float(n);
    if (p > 0.f) h -= p * log2f(p);
  }
  if (lane == 0) entropy[v] = h;
}

// One CTA per pair (x, y): the joint probabilities of all bin pairs
// (get_mi, inst/cuda/mi.cu:115-152) and MI = sum p log2 p + H(x) + H(y).
__global__ void __launch_bounds__(128)
mi_pair_kernel(const float *__restrict__ wx, const float *__restrict__ wy, int64_t nx, int64_t ny,
               int64_t n, int nbins, const float *__restrict__ hx, const float *__restrict__ hy,
               float *__restrict__ out) {
  const int64_t x = blockIdx.x, y = blockIdx.y;
  const float *a0 = wx + x * nbins * n, *b0 = wy + y * nbins * n;
  float sum = 0.f;
  for (int cell = threadIdx.x; cell < nbins * nbins; cell += blockDim.x) {
    const float *a = a0 + (cell / nbins) * n, *b = b0 + (cell % nbins) * n;
    float s = 0.f;
    for (int64_t k = 0; k < n; k++) s = fmaf(a[k], b[k], s);
    const float p = s / float(n);
    if (p > 0.f) sum += p * __log2f(p);
  }
  __shared__ float red[4];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) out[y * nx + x] = red[0] + red[1] + red[2] + red[3] + hx[x] + hy[y];
}

template <int ORDER>
void launch_prep(const float *X, int64_t nvar, int64_t n, int nbins, int lg, int64_t kpad,
                 uint16_t *planes, float *wts, float *entropy, cudaStream_t s) {
  mi_prep_kernel<ORDER><<<unsigned(cdiv(nvar, 8)), 256, 0, s>>>(X, nvar, n, nbins, lg, kpad,
                                                                planes, wts, entropy);
}

int prep(int order, const float *X, int64_t nvar, int64_t n, int nbins, int lg, int64_t kpad,
         uint16_t *planes, float *wts, float *entropy, cudaStream_t s) {
  switch (order) {
    case 1: launch_prep<1>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 2: launch_prep<2>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 3: launch_prep<3>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 4: launch_prep<4>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 5: launch_prep<5>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 6: launch_prep<6>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    case 7: launch_prep<7>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
    default: launch_prep<8>(X, nvar, n, nbins, lg, kpad, planes, wts, entropy, s); break;
  }
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

int mi_check(int nbins, int order, int64_t n, int64_t nx, int64_t ny) {
  if (nbins < 1) return fail(GT_EINVAL, "bins must be at least 1");
  if (order < 1 || order > nbins || order > kMiMaxOrder)
    return fail(GT_EINVAL, "splineOrder must lie in 1 .. min(bins, %d)", kMiMaxOrder);
  if (n < 1) return fail(GT_EINVAL, "need at least one sample");
  if (nx < 0 || ny < 0) return fail(GT_EINVAL, "negative size");
  if (nx > 65535 * 8 || ny > 65535) return fail(GT_EINVAL, "too many variables");
  return GT_OK;
}

}  // namespace

int mi_impl(int nbins, int order, int64_t n, const float *dX, int64_t nx, const float *dY,
            int64_t ny, float *dOut, cudaStream_t s) {
  GT_TRY(mi_check(nbins, order, n, nx, ny));
  if (nx == 0 || ny == 0) return GT_OK;
  const bool sym = dX == dY && nx == ny;
  const bool tc = nbins <= kMiMaxTcBins && gt_get_gram_path() != GT_GRAM_FP32;
  void *ph = nullptr;
  GT_TRY(ws_get(WS_SCRATCH2, size_t(nx + ny) * sizeof(float), &ph));
  float *hx = static_cast<float *>(ph), *hy = sym ? hx : hx + nx;
  if (tc) {
    int lg = 0;
    while ((1 << lg) < nbins) lg++;
    const int64_t nbp = int64_t(1) << lg, kpad = cdiv(n, 64) * 64;
    const size_t bx = size_t(2) * size_t(nx * nbp) * size_t(kpad) * 2;
    const size_t by = sym ? 0 : size_t(2) * size_t(ny * nbp) * size_t(kpad) * 2;
    void *pp = nullptr;
    GT_TRY(ws_get(WS_SCRATCH0, bx + by, &pp));
    auto *px = static_cast<uint16_t *>(pp);
    auto *py = sym ? px : px + bx / 2;
    {
      ProfScope prof("mi_prologue", s);
      GT_TRY(prep(order, dX, nx, n, nbins, lg, kpad, px, nullptr, hx, s));
      if (!sym) GT_TRY(prep(order, dY, ny, n, nbins, lg, kpad, py, nullptr, hy, s));
    }
    return mi_tc(px, nx * nbp, py, ny * nbp, kpad, lg, nbins, nx, ny, n, hx, hy, dOut, sym ? 1 : 0,
                 s);
  }
  const size_t wx = size_t(nx) * size_t(nbins) * size_t(n) * 4;
  const size_t wy = sym ? 0 : size_t(ny) * size_t(nbins) * size_t(n) * 4;
  void *pw = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, wx + wy, &pw));
  auto *fx = static_cast<float *>(pw);
  auto *fy = sym ? fx : fx + wx / 4;
  ProfScope prof("mi_pairs", s);
  GT_TRY(prep(order, dX, nx, n, nbins, 0, 0, nullptr, fx, nullptr, s));
  mi_entropy_kernel<<<unsigned(cdiv(nx, 8)), 256, 0, s>>>(fx, nx, n, nbins, hx);
  count_launch();
  if (!sym) {
    GT_TRY(prep(order, dY, ny, n, nbins, 0, 0, nullptr, fy, nullptr, s));
    mi_entropy_kernel<<<unsigned(cdiv(ny, 8)), 256, 0, s>>>(fy, ny, n, nbins, hy);
    count_launch();
  }
  mi_pair_kernel<<<dim3(unsigned(nx), unsigned(ny)), 128, 0, s>>>(fx, fy, nx, ny, n, nbins, hx,
                                                                  hy, dOut);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_mutual_info_device(int nbins, int order, int64_t n, const float *d_X,
                                     int64_t nx, const float *d_Y, int64_t ny, float *d_out,
                                     void *stream) {
  gt::clear_error();
  if ((nx > 0 && !d_X) || (ny > 0 && !d_Y) || (nx > 0 && ny > 0 && !d_out))
    return gt::fail(GT_EINVAL, "null device pointer");
  return gt::mi_impl(nbins, order, n, d_X, nx, d_Y, ny, d_out, static_cast<cudaStream_t>(stream));
}

extern "C" int gt_mutual_info(int nbins, int order, int64_t n, const float *X, int64_t nx,
                              const float *Y, int64_t ny, float *out) {
  gt::clear_error();
  GT_TRY(gt::mi_check(nbins, order, n, nx, ny));
  if (nx == 0 || ny == 0) return GT_OK;
  if (!X || !Y || !out) return gt::fail(GT_EINVAL, "null host pointer");
  cudaStream_t s = gt::lib_stream();
  gt::StreamSyncGuard guard(s);
  const size_t bx = size_t(nx) * size_t(n) * 4, by = size_t(ny) * size_t(n) * 4;
  const size_t bo = size_t(nx) * size_t(ny) * 4;
  const bool sym = X == Y && nx == ny;
  void *dx = nullptr, *dy = nullptr, *dout = nullptr;
  GT_TRY(gt::ws_get(gt::WS_IN_A, bx, &dx));
  GT_CUDA(cudaMemcpyAsync(dx, X, bx, cudaMemcpyHostToDevice, s));
  if (!sym) {
    GT_TRY(gt::ws_get(gt::WS_IN_B, by, &dy));
    GT_CUDA(cudaMemcpyAsync(dy, Y, by, cudaMemcpyHostToDevice, s));
  } else {
    dy = dx;
  }
  GT_TRY(gt::ws_get(gt::WS_OUT0, bo, &dout));
  GT_TRY(gt::mi_impl(nbins, order, n, static_cast<float *>(dx), nx, static_cast<float *>(dy), ny,
                     static_cast<float *>(dout), s));
  GT_CUDA(cudaMemcpyAsync(out, dout, bo, cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  bool failed = false;
  GT_TRY(gt::device_error_check(s, &failed));
  if (failed) return gt::fail(GT_ETIMEOUT, "a tensor-core kernel wait timed out");
  return GT_OK;
}
