// correlation.cu -- gpuCor(method = "pearson") and gpuTtest.
//
// Reference: src/correlation.cpp:66-161 pmcc() runs three per-pair kernels
// (inst/cuda/correlation.cu:7-292: means -> standard deviations -> sum of
// z-score products), each one block per (x, y) pair that re-reads both
// columns, stores O(nA*nB) temporary means/SDs, and computes t-scores on the
// host (hostSignif, src/correlation.cpp:51-64).
//
// Here:
//  * a prologue computes each variable's mean and norm once, in FP64
//    (corrected two-pass), and writes the normalised column
//    z = (x - mean) / ||x - mean||, so r(x, y) = <z_x, z_y>;
//  * "everything": the Gram contraction runs on tcgen05 tensor cores
//    (split bf16, gram_tc.cu) or, for GT_GRAM_FP32, on the CUDA-core engine;
//  * "pairwise.complete.obs": on inputs without a missing value it is the
//    "everything" result, so that tensor-core path runs (gated on a device
//    NaN flag); otherwise the masked tensor-core Gram (pairwise_tc.cu) forms
//    the six sums per pair (count, sums, squares, cross); the FP32 path
//    accumulates them on the CUDA-core engine; r comes from them in FP64;
//  * pairs, r and the t-score (hostSignif's rule, in float as the reference
//    evaluates it) are written by the same epilogue; cor(x) computes each
//    unordered pair once and mirrors it.
#include "common.cuh"
#include "allpairs_simt.cuh"
#include "kernels.cuh"
#include "stats.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace gt {

namespace {

constexpr int kStatThreads = 256;  // eight variables per CTA, one warp each

__global__ void __launch_bounds__(kStatThreads)
colstats_kernel(const float *__restrict__ X, int64_t nvar, int64_t n, int use,
                ColStats *__restrict__ out, const int *run_if = nullptr) {
  if (run_if && *run_if == 0) return;  // a gated launch whose gate is closed
  const int64_t v = (int64_t(blockIdx.x) * kStatThreads + threadIdx.x) >> 5;
  if (v >= nvar) return;  // whole warps
  const ColStats st = colstats_warp(X + v * n, n, use);
  if ((threadIdx.x & 31) == 0) out[v] = st;
}

// z[v][k] = (x - mean) * inv_norm in float, rows of length ldz (>= n, pad
// filled with `padv`), one CTA per variable.  Everything mode: a variable
// containing NaN or with zero variance becomes all-NaN, so every r involving
// it is NaN.
__global__ void normalize_f32_kernel(const float *__restrict__ X, int64_t nvar, int64_t n,
                                     int64_t ldz, const ColStats *__restrict__ st, int use,
                                     float padv, float *__restrict__ Z,
                                     const int *run_if = nullptr) {
  if (run_if && *run_if == 0) return;  // a gated launch whose gate is closed
  const int64_t v = blockIdx.x;
  const ColStats s = st[v];
  const Centerer cen(s);
  const float *x = X + v * n;
  float *z = Z + v * ldz;
  for (int64_t k = threadIdx.x; k < ldz; k += blockDim.x) {
    float val;
    if (k >= n) val = padv;
    else if (use == 0 && s.flags) val = __int_as_float(0x7fc00000);
    else val = cen(x[k]);
    z[k] = val;
  }
}

__device__ __forceinline__ float clamp_r(float r) { return r > 1.f ? 1.f : (r < -1.f ? -1.f : r); }

// hostSignif (src/correlation.cpp:51-64), evaluated in float as there.
__device__ __forceinline__ float signif(float r, float pairs) {
  if (r >= 0.999f) return 10000.0f;
  return r * sqrtf((pairs - 2.f) / (1.f - r * r));
}

struct OpDot {
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const { c[0] = fmaf(a, b, c[0]); }
};

struct OutPearsonF32 {
  PearsonOut o;
  __device__ void operator()(int64_t r, int64_t c, const float (&acc)[1], bool mirror) const {
    float v = clamp_r(acc[0]);
    if (o.symmetric && r == c && v == v) v = 1.f;
    const float t = signif(v, o.npairs);
    const int64_t i0 = r * o.ld + c, i1 = c * o.ld + r;
    if (o.corr) { o.corr[i0] = v; if (mirror) o.corr[i1] = v; }
    if (o.ts) { o.ts[i0] = t; if (mirror) o.ts[i1] = t; }
    if (o.pairs) { o.pairs[i0] = o.npairs; if (mirror) o.pairs[i1] = o.npairs; }
  }
};

// Pairwise-complete sums over observations where both values are present:
// count, sum a, sum b, sum a^2, sum b^2, sum a*b.
struct OpPairwise {
  static constexpr int NACC = 6;
  static constexpr int kUnrollK = 4;  // 3 % faster than a full unroll
  __device__ static float pad() { return __int_as_float(0x7fc00000); }
  __device__ void init(float (&c)[6]) const {
#pragma unroll
    for (int i = 0; i < 6; i++) c[i] = 0.f;
  }
  __device__ void step(float (&c)[6], float a, float b) const {
    const bool both = (a == a) & (b == b);
    const float fa = both ? a : 0.f, fb = both ? b : 0.f;
    c[0] += both ? 1.f : 0.f;
    c[1] += fa;
    c[2] += fb;
    c[3] = fmaf(fa, fa, c[3]);
    c[4] = fmaf(fb, fb, c[4]);
    c[5] = fmaf(fa, fb, c[5]);
  }
};

struct OutPairwise {
  PearsonOut o;
  __device__ void operator()(int64_t r, int64_t c, const float (&acc)[6], bool mirror) const {
    const double n = acc[0];
    float v = __int_as_float(0x7fc00000);
    if (n >= 2.0) {
      const double sa = acc[1], sb = acc[2];
      const double va = double(acc[3]) - sa * sa / n;
      const double vb = double(acc[4]) - sb * sb / n;
      const double cv = double(acc[5]) - sa * sb / n;
      if (va > 0.0 && vb > 0.0) v = clamp_r(float(cv / sqrt(va * vb)));
    }
    if (o.symmetric && r == c && v == v) v = 1.f;
    const float np = float(n);
    const float t = signif(v, np);
    const int64_t i0 = r * o.ld + c, i1 = c * o.ld + r;
    if (o.corr) { o.corr[i0] = v; if (mirror) o.corr[i1] = v; }
    if (o.ts) { o.ts[i0] = t; if (mirror) o.ts[i1] = t; }
    if (o.pairs) { o.pairs[i0] = np; if (mirror) o.pairs[i1] = np; }
  }
};

__global__ void ttest_kernel(const float *__restrict__ pairs, const float *__restrict__ r,
                             int64_t n, float *__restrict__ ts) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float c = r[i];
    ts[i] = c * sqrtf((pairs[i] - 2.f) / (1.f - c * c));
  }
}

__global__ void differ_kernel(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                              int64_t nwords, int *flag) {
  int local = 0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nwords;
       i += int64_t(gridDim.x) * blockDim.x)
    local |= (a[i] != b[i]);
  if (__syncthreads_or(local) && threadIdx.x == 0) atomicOr(flag, 1);
}

// flag |= 1 if any of x[0..count) is NaN.
__global__ void any_nan_kernel(const float *__restrict__ x, int64_t count, int *flag) {
  int local = 0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count;
       i += int64_t(gridDim.x) * blockDim.x)
    local |= (x[i] != x[i]);
  if (__syncthreads_or(local) && threadIdx.x == 0) atomicOr(flag, 1);
}

int grid_for(int64_t work, int threads) {
  const int64_t g = cdiv(work, threads);
  const int64_t cap = int64_t(sm_count()) * 16;
  return int(g < 1 ? 1 : (g > cap ? cap : g));
}

// Column statistics + normalised float rows for one operand.
int prologue_f32(const float *dX, int64_t nvar, int64_t n, int use, int64_t ldz, int slot_z,
                 int slot_st, float **Z, ColStats **st, cudaStream_t s,
                 const int *run_if = nullptr) {
  void *pz = nullptr, *pst = nullptr;
  GT_TRY(ws_get(slot_z, size_t(nvar) * size_t(ldz) * 4, &pz));
  GT_TRY(ws_get(slot_st, size_t(nvar) * sizeof(ColStats), &pst));
  *Z = static_cast<float *>(pz);
  *st = static_cast<ColStats *>(pst);
  ProfScope prof("pearson_prologue", s);
  colstats_kernel<<<unsigned(cdiv(nvar, kStatThreads / 32)), kStatThreads, 0, s>>>(dX, nvar, n, use,
                                                                                 *st, run_if);
  count_launch();
  const float padv = use == 0 ? 0.f : __builtin_nanf("");
  normalize_f32_kernel<<<unsigned(nvar), 256, 0, s>>>(dX, nvar, n, ldz, *st, use, padv, *Z,
                                                      run_if);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

// Device flag (bytes 128..131 of the small scratch slot): 1 if a or b holds
// a NaN.  Asynchronous on s.
int any_nan_flag(const float *a, int64_t na, const float *b, int64_t nb, int **flag,
                 cudaStream_t s) {
  void *pf = nullptr;
  GT_TRY(ws_get(WS_SCRATCH4, 256, &pf));
  *flag = static_cast<int *>(pf) + 32;
  GT_CUDA(cudaMemsetAsync(*flag, 0, sizeof(int), s));
  if (na > 0) {
    any_nan_kernel<<<grid_for(na, 256), 256, 0, s>>>(a, na, *flag);
    count_launch();
  }
  if (b && nb > 0) {
    any_nan_kernel<<<grid_for(nb, 256), 256, 0, s>>>(b, nb, *flag);
    count_launch();
  }
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

}  // namespace

// Column statistics (FP64 mean, inverse norm, flags) of nvar variables.
int launch_colstats(const float *dX, int64_t nvar, int64_t n, int use, ColStats *st,
                    cudaStream_t s) {
  if (nvar == 0) return GT_OK;
  if (nvar > 2147483647LL) return fail(GT_EINVAL, "too many variables");
  colstats_kernel<<<unsigned(cdiv(nvar, kStatThreads / 32)), kStatThreads, 0, s>>>(dX, nvar, n, use,
                                                                                 st);
  count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

// prologue for the tensor-core path lives in gram_tc.cu
int pearson_tc_prologue(const float *dX, int64_t nvar, int64_t n, int kind, int slot_z,
                        int slot_st, void **Z, int64_t *kpad, cudaStream_t s);

int pearson_impl(int use, const float *dA, int64_t nA, const float *dB, int64_t nB, int64_t n,
                 float *pairs, float *corr, float *ts, int symmetric, cudaStream_t s) {
  if (nA == 0 || nB == 0) return GT_OK;
  PearsonOut po{corr, ts, pairs, nB, float(n), symmetric};
  const int path = gt_get_gram_path();
  const bool tc = path != GT_GRAM_FP32 && n > 0;
  // pairwise.complete.obs on inputs without a missing value is cor(everything):
  // a device flag (any NaN in A or B) gates two launches, the tensor-core
  // Gram of everything mode (runs if the flag is clear) and the masked
  // tensor-core Gram (runs if it is set), so the call stays asynchronous.
  // The FP32 path keeps the CUDA-core six-sum kernel
  int *nan_flag = nullptr;
  if (use != GT_EVERYTHING && tc) {
    GT_TRY(any_nan_flag(dA, nA * n, symmetric ? nullptr : dB, nB * n, &nan_flag, s));
    po.gate = nan_flag;
  }
  if (tc) {
    void *zA = nullptr, *zB = nullptr;
    int64_t kpad = 0;
    GT_TRY(pearson_tc_prologue(dA, nA, n, path, WS_SCRATCH0, WS_SCRATCH2, &zA, &kpad, s));
    if (symmetric) zB = zA;
    else GT_TRY(pearson_tc_prologue(dB, nB, n, path, WS_SCRATCH1, WS_SCRATCH3, &zB, &kpad, s));
    GT_TRY(pearson_tc(zA, nA, zB, nB, kpad, path, po, s));
    if (use == GT_EVERYTHING) return GT_OK;
    // with a missing value: the masked tensor-core Gram (pairwise_tc.cu)
    return pearson_pairwise_tc(dA, nA, symmetric ? dA : dB, nB, n, po, nan_flag, s);
  }
  const int64_t ldz = (n + 3) / 4 * 4;
  float *zA = nullptr, *zB = nullptr;
  ColStats *sA = nullptr, *sB = nullptr;
  GT_TRY(prologue_f32(dA, nA, n, use, ldz, WS_SCRATCH0, WS_SCRATCH2, &zA, &sA, s, nan_flag));
  if (symmetric) zB = zA;
  else GT_TRY(prologue_f32(dB, nB, n, use, ldz, WS_SCRATCH1, WS_SCRATCH3, &zB, &sB, s, nan_flag));
  SimtArgs a;
  a.R = zA; a.C = zB;
  a.ldr = a.ldc = ldz;
  a.nr = nA; a.nc = nB;
  a.K = ldz;
  a.symmetric = symmetric;
  a.vec_ok = 1;
  a.run_if = nan_flag;
  cudaError_t e;
  ProfScope prof(use == GT_EVERYTHING ? "pearson_gram" : "pearson_pairwise", s);
  if (use == GT_EVERYTHING) {
    const int64_t t = cdiv(nA, 128) * cdiv(nB, 128) / (symmetric ? 2 : 1);
    if (t >= 2 * sm_count())
      e = launch_allpairs_simt<OpDot, OutPearsonF32, 8, 8>(a, OpDot{}, OutPearsonF32{po}, s);
    else
      e = launch_allpairs_simt<OpDot, OutPearsonF32, 4, 4>(a, OpDot{}, OutPearsonF32{po}, s);
  } else {
    e = launch_allpairs_simt<OpPairwise, OutPairwise, 4, 4>(a, OpPairwise{}, OutPairwise{po}, s);
  }
  if (e != cudaSuccess) return fail(GT_ECUDA, "pearson kernel launch: %s", cudaGetErrorString(e));
  return GT_OK;
}

int pearson_check(int use, int64_t nA, int64_t nB, int64_t n) {
  if (use != GT_EVERYTHING && use != GT_PAIRWISE_COMPLETE)
    return fail(GT_EINVAL, "unknown use method");
  if (nA < 0 || nB < 0 || n < 0) return fail(GT_EINVAL, "negative size");
  if (nA > 2147483647LL || nB > 2147483647LL) return fail(GT_EINVAL, "too many variables");
  if (cdiv(nA, 64) > 65535) return fail(GT_EINVAL, "too many variables (%lld)", (long long)nA);
  return GT_OK;
}

// Device-side equality of two float buffers (bitwise), used to recognise
// gpuCor(x) called through .C, which always passes two copies of x.
int same_contents(const float *a, const float *b, int64_t count, bool *same, cudaStream_t s) {
  void *pf = nullptr;
  GT_TRY(ws_get(WS_SCRATCH4, 256, &pf));
  int *flag = static_cast<int *>(pf);
  GT_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
  if (count > 0)
    differ_kernel<<<grid_for(count, 256), 256, 0, s>>>(reinterpret_cast<const uint32_t *>(a),
                                                        reinterpret_cast<const uint32_t *>(b),
                                                        count, flag);
  if (count > 0) count_launch();
  int h = 1;
  GT_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  *same = (h == 0);
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_pmcc_device(int use, const float *d_A, int64_t nA, const float *d_B, int64_t nB,
                              int64_t n, float *d_pairs, float *d_corr, float *d_ts,
                              void *stream) {
  gt::clear_error();
  GT_TRY(gt::pearson_check(use, nA, nB, n));
  if ((nA > 0 && !d_A) || (nB > 0 && !d_B)) return gt::fail(GT_EINVAL, "null device pointer");
  const int sym = (d_A == d_B && nA == nB) ? 1 : 0;
  return gt::pearson_impl(use, d_A, nA, d_B, nB, n, d_pairs, d_corr, d_ts, sym,
                          static_cast<cudaStream_t>(stream));
}

namespace gt {
namespace {

// Matrices from this size on (floats; 256 MB) have their constant pair counts
// filled on the host: with 16 threads the fill hides behind the link time of
// the other two matrices; below it, the device writing one more matrix over
// the link is the cheaper way.
constexpr int64_t kHostFillMin = int64_t(64) << 20;

// Writes v into out[0 .. count) with up to 16 host threads.
void host_fill(float *out, int64_t count, float v) {
  const int64_t per = int64_t(4) << 20;  // floats per thread, at least
  int64_t nt = (count + per - 1) / per;
  const int64_t hw = std::max<int64_t>(1, std::thread::hardware_concurrency());
  nt = std::min<int64_t>(std::min<int64_t>(nt, 16), hw);
  if (nt <= 1) {
    std::fill_n(out, count, v);
    return;
  }
  // slices that get no thread (thread creation failed) are filled here
  std::vector<std::thread> th;
  int64_t done = 0;
  try {
    th.reserve(size_t(nt));
    for (int64_t t = 0; t < nt; t++) {
      const int64_t b = count * t / nt, e = count * (t + 1) / nt;
      th.emplace_back([=] { std::fill_n(out + b, e - b, v); });
      done = e;
    }
  } catch (...) {
  }
  std::fill_n(out + done, count - done, v);
  for (auto &x : th) x.join();
}

}  // namespace
}  // namespace gt

namespace gt {
namespace {

// Outputs from this size on (bytes per matrix; 64 MB) that the kernels cannot
// write in place (pageable memory, as R's .C passes) go through the banded
// pipeline below when the Gram path supports it.
constexpr size_t kBandMinBytes = size_t(64) << 20;
constexpr int kBands = 16;

// "everything" Pearson into host outputs the kernels cannot write in place
// (pageable memory): the Gram runs in kBands bands of rows
// (pearson_band_tiles; once band b has run, its rows are complete, mirror
// entries included) into device workspace, and each band's rows go to the
// caller's buffers by a device-to-host copy on a second stream as soon as the
// band's event completes, while the device computes the next bands.  The copy
// of a whole matrix after the computation (measured at 4096 x 20000, f16x6:
// 31 ms per call) then overlaps it instead; the constant pair counts are
// filled by host threads meanwhile.  (Kernels writing page-locked staging
// with host threads copying it out measured slower, 41 ms: the host copies
// and the fill share the host's memory bandwidth and cores.)
int pmcc_banded(const float *dA, int64_t nA, const float *dB, int64_t nB, int64_t n, int sym,
                int path, float *pairs, float *corr, float *ts, cudaStream_t s) {
  const size_t outb = size_t(nA) * size_t(nB) * 4;
  float *c_dev = corr ? static_cast<float *>(host_direct_ptr(corr)) : nullptr;
  float *t_dev = ts ? static_cast<float *>(host_direct_ptr(ts)) : nullptr;
  const bool stage_c = corr && !c_dev, stage_t = ts && !t_dev;
  void *o0 = nullptr, *o1 = nullptr;
  if (stage_c) GT_TRY(ws_get(WS_OUT0, outb, &o0));
  if (stage_t) GT_TRY(ws_get(WS_OUT1, outb, &o1));
  if (stage_c) c_dev = static_cast<float *>(o0);
  if (stage_t) t_dev = static_cast<float *>(o1);
  // operand planes, then the bands
  void *zA = nullptr, *zB = nullptr;
  int64_t kpad = 0;
  GT_TRY(pearson_tc_prologue(dA, nA, n, path, WS_SCRATCH0, WS_SCRATCH2, &zA, &kpad, s));
  if (sym) zB = zA;
  else GT_TRY(pearson_tc_prologue(dB, nB, n, path, WS_SCRATCH1, WS_SCRATCH3, &zB, &kpad, s));
  const int64_t tr = cdiv(nA, kGramRows);
  const int64_t band_blocks = cdiv(tr, kBands);
  std::vector<int2> tiles;
  std::vector<int64_t> off;
  pearson_band_tiles(nA, nB, sym != 0, band_blocks, tiles, off);
  const int64_t nbands = int64_t(off.size()) - 1;
  void *dt = nullptr;
  GT_TRY(ws_get(WS_TILES, tiles.size() * sizeof(int2), &dt));
  GT_CUDA(cudaMemcpyAsync(dt, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
  struct Resources {
    std::vector<cudaEvent_t> ev;
    cudaStream_t cs = nullptr;
    ~Resources() {
      if (cs) {
        cudaStreamSynchronize(cs);
        cudaStreamDestroy(cs);
      }
      for (auto x : ev)
        if (x) cudaEventDestroy(x);
    }
  } res;
  res.ev.assign(size_t(nbands), nullptr);
  for (auto &e : res.ev) GT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  GT_CUDA(cudaStreamCreateWithFlags(&res.cs, cudaStreamNonBlocking));
  PearsonOut po{c_dev, t_dev, nullptr, nB, float(n), sym};
  for (int64_t b = 0; b < nbands; b++) {
    GT_TRY(pearson_tc_band(zA, nA, zB, nB, kpad, path, po, static_cast<const int2 *>(dt) + off[b],
                           off[b + 1] - off[b], s));
    GT_CUDA(cudaEventRecord(res.ev[size_t(b)], s));
  }
  // the pair counts on host threads while the bands run and are copied
  std::thread filler;
  bool filler_started = false;
  if (pairs) {
    try {
      filler = std::thread([=] { host_fill(pairs, nA * nB, float(n)); });
      filler_started = true;
    } catch (...) {
    }
  }
  const int64_t rows_per_band = band_blocks * kGramRows;
  int st = GT_OK;
  for (int64_t b = 0; b < nbands && st == GT_OK; b++) {
    const int64_t r0 = b * rows_per_band, r1 = std::min(nA, r0 + rows_per_band);
    const size_t e0 = size_t(r0) * size_t(nB), bytes = size_t(r1 - r0) * size_t(nB) * 4;
    cudaError_t e = cudaStreamWaitEvent(res.cs, res.ev[size_t(b)], 0);
    if (e == cudaSuccess && stage_c)
      e = cudaMemcpyAsync(corr + e0, c_dev + e0, bytes, cudaMemcpyDeviceToHost, res.cs);
    if (e == cudaSuccess && stage_t)
      e = cudaMemcpyAsync(ts + e0, t_dev + e0, bytes, cudaMemcpyDeviceToHost, res.cs);
    if (e != cudaSuccess) st = fail(GT_ECUDA, "banded Pearson copy: %s", cudaGetErrorString(e));
  }
  if (st == GT_OK) {
    cudaError_t e = cudaStreamSynchronize(res.cs);
    if (e != cudaSuccess) st = fail(GT_ECUDA, "banded Pearson copy: %s", cudaGetErrorString(e));
  }
  if (filler_started) filler.join();
  else if (pairs) host_fill(pairs, nA * nB, float(n));
  return st;
}

}  // namespace
}  // namespace gt

extern "C" int gt_pmcc(int use, const float *A, int64_t nA, const float *B, int64_t nB, int64_t n,
                       float *pairs, float *corr, float *ts) {
  gt::clear_error();
  GT_TRY(gt::pearson_check(use, nA, nB, n));
  if (nA == 0 || nB == 0) return GT_OK;
  if (!A || !B) return gt::fail(GT_EINVAL, "null host pointer");
  cudaStream_t s = gt::lib_stream();
  gt::StreamSyncGuard guard(s);
  const size_t inA = size_t(nA) * size_t(n) * 4, inB = size_t(nB) * size_t(n) * 4;
  const size_t outb = size_t(nA) * size_t(nB) * 4;
  void *dA = nullptr, *dB = nullptr, *o0 = nullptr, *o1 = nullptr, *o2 = nullptr;
  GT_TRY(gt::ws_get(gt::WS_IN_A, inA, &dA));
  GT_CUDA(cudaMemcpyAsync(dA, A, inA, cudaMemcpyHostToDevice, s));
  bool sym = (A == B && nA == nB);
  if (!sym) {
    GT_TRY(gt::ws_get(gt::WS_IN_B, inB, &dB));
    GT_CUDA(cudaMemcpyAsync(dB, B, inB, cudaMemcpyHostToDevice, s));
    if (nA == nB)
      GT_TRY(gt::same_contents(static_cast<float *>(dA), static_cast<float *>(dB), nA * n, &sym, s));
  }
  if (sym) dB = dA;
  const int path = gt_get_gram_path();
  if (use == GT_EVERYTHING && n > 0 && outb >= gt::kBandMinBytes &&
      (path == GT_GRAM_TC_F16X3 || path == GT_GRAM_TC_F16X6) &&
      ((corr && !gt::host_direct_ptr(corr)) || (ts && !gt::host_direct_ptr(ts)))) {
    GT_TRY(gt::pmcc_banded(static_cast<float *>(dA), nA, static_cast<float *>(dB), nB, n,
                           sym ? 1 : 0, path, pairs, corr, ts, s));
    GT_CUDA(cudaStreamSynchronize(s));
    bool failed = false;
    GT_TRY(gt::device_error_check(s, &failed));
    if (failed) return gt::fail(GT_ETIMEOUT, "a tensor-core kernel wait timed out");
    return GT_OK;
  }
  // "everything": every pair count is n (src/correlation.cpp:66-161 counts
  // all observations), so for large outputs the host fills `pairs` while the
  // device works and the host link carries two matrices instead of three
  const bool host_pairs = pairs && use == GT_EVERYTHING && nA * nB >= gt::kHostFillMin;
  // outputs the kernels can write in place (no staging copy), else workspace
  void *h0 = corr ? gt::host_output_ptr(corr, outb) : nullptr;
  void *h1 = ts ? gt::host_output_ptr(ts, outb) : nullptr;
  void *h2 = pairs && !host_pairs ? gt::host_output_ptr(pairs, outb) : nullptr;
  if (corr && !(o0 = h0)) GT_TRY(gt::ws_get(gt::WS_OUT0, outb, &o0));
  if (ts && !(o1 = h1)) GT_TRY(gt::ws_get(gt::WS_OUT1, outb, &o1));
  if (pairs && !host_pairs && !(o2 = h2)) GT_TRY(gt::ws_get(gt::WS_OUT2, outb, &o2));
  GT_TRY(gt::pearson_impl(use, static_cast<float *>(dA), nA, static_cast<float *>(dB), nB, n,
                          static_cast<float *>(o2), static_cast<float *>(o0),
                          static_cast<float *>(o1), sym ? 1 : 0, s));
  if (corr && !h0) GT_CUDA(cudaMemcpyAsync(corr, o0, outb, cudaMemcpyDeviceToHost, s));
  if (ts && !h1) GT_CUDA(cudaMemcpyAsync(ts, o1, outb, cudaMemcpyDeviceToHost, s));
  if (pairs && !host_pairs && !h2)
    GT_CUDA(cudaMemcpyAsync(pairs, o2, outb, cudaMemcpyDeviceToHost, s));
  if (host_pairs) gt::host_fill(pairs, nA * nB, float(n));
  GT_CUDA(cudaStreamSynchronize(s));
  bool failed = false;
  GT_TRY(gt::device_error_check(s, &failed));
  if (failed) return gt::fail(GT_ETIMEOUT, "a tensor-core kernel wait timed out");
  return GT_OK;
}

extern "C" int gt_ttest_device(const float *d_pairs, const float *d_coeffs, int64_t n, float *d_ts,
                               void *stream) {
  gt::clear_error();
  if (n < 0) return gt::fail(GT_EINVAL, "negative size");
  if (n == 0) return GT_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gt::ttest_kernel<<<gt::grid_for(n, 256), 256, 0, s>>>(d_pairs, d_coeffs, n, d_ts);
  gt::count_launch();
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free Pearson.
//
// Some callers cannot let a library allocate device memory: processes whose
// device memory is owned by another allocator (a framework's caching
// allocator, or a fixed per-process budget) where a cudaMalloc made behind
// their back fails or breaks their accounting, and latency-sensitive callers
// that cannot afford the device-wide synchronisation cudaMalloc/cudaFree may
// bring.  gt_pmcc_device_noalloc serves them: it runs the FP32 CUDA-core
// Pearson path with its scratch (normalised rows and column statistics) in
// the file-scope array below, which every device that loads the library
// holds until the process exits.
namespace gt {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
int noalloc_scratch(unsigned char **out) {
  int dev = 0;
  GT_TRY(current_device(&dev));
  if (dev >= kNoAllocMaxDevices) return fail(GT_ENODEV, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(GT_ECUDA, "cudaGetSymbolAddress(g_noalloc_scratch) failed: %s",
                  cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_noalloc_addr[dev]);
  return GT_OK;
}

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace
}  // namespace gt

extern "C" int gt_pmcc_device_noalloc(int use, const float *d_A, int64_t nA, const float *d_B,
                                      int64_t nB, int64_t n, float *d_pairs, float *d_corr,
                                      float *d_ts, void *stream) {
  using namespace gt;
  clear_error();
  GT_TRY(pearson_check(use, nA, nB, n));
  if ((nA > 0 && !d_A) || (nB > 0 && !d_B)) return fail(GT_EINVAL, "null device pointer");
  if (nA == 0 || nB == 0) return GT_OK;
  const bool sym = (d_A == d_B && nA == nB);
  // one normalised row alone must fit; this also keeps the size products
  // below from wrapping (nA, nB < 2^31 and n < 2^24)
  if (n > int64_t(kNoAllocScratchBytes / 4))
    return fail(GT_EINVAL,
                "gt_pmcc_device_noalloc: %lld observations exceed the %zu bytes of scratch of "
                "the allocation-free entry point; use gt_pmcc_device",
                (long long)n, kNoAllocScratchBytes);
  const int64_t ldz = (n + 3) / 4 * 4;
  // scratch layout: zA | zB (two sets only) | statsA | statsB
  const size_t bzA = round256(size_t(nA) * size_t(ldz) * 4);
  const size_t bzB = sym ? 0 : round256(size_t(nB) * size_t(ldz) * 4);
  const size_t bsA = round256(size_t(nA) * sizeof(ColStats));
  const size_t bsB = sym ? 0 : round256(size_t(nB) * sizeof(ColStats));
  const size_t need = bzA + bzB + bsA + bsB;
  if (need > kNoAllocScratchBytes)
    return fail(GT_EINVAL,
                "gt_pmcc_device_noalloc: this problem needs %zu bytes of scratch but the "
                "allocation-free entry point has %zu (nA=%lld, nB=%lld, n=%lld); use "
                "gt_pmcc_device",
                need, kNoAllocScratchBytes, (long long)nA, (long long)nB, (long long)n);
  unsigned char *base = nullptr;
  GT_TRY(noalloc_scratch(&base));
  float *zA = reinterpret_cast<float *>(base);
  float *zB = sym ? zA : reinterpret_cast<float *>(base + bzA);
  ColStats *sA = reinterpret_cast<ColStats *>(base + bzA + bzB);
  ColStats *sB = sym ? sA : reinterpret_cast<ColStats *>(base + bzA + bzB + bsA);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Every scratch byte read below is written first in the same call (all ldz
  // entries of each row, every statistic), so nothing has to be cleared.
  const float padv = use == GT_EVERYTHING ? 0.f : __builtin_nanf("");
  GT_TRY(launch_colstats(d_A, nA, n, use, sA, s));
  normalize_f32_kernel<<<unsigned(nA), 256, 0, s>>>(d_A, nA, n, ldz, sA, use, padv, zA);
  count_launch();
  if (!sym) {
    GT_TRY(launch_colstats(d_B, nB, n, use, sB, s));
    normalize_f32_kernel<<<unsigned(nB), 256, 0, s>>>(d_B, nB, n, ldz, sB, use, padv, zB);
    count_launch();
  }
  GT_CUDA(cudaGetLastError());
  PearsonOut po{d_corr, d_ts, d_pairs, nB, float(n), sym ? 1 : 0};
  SimtArgs a;
  a.R = zA; a.C = zB;
  a.ldr = a.ldc = ldz;
  a.nr = nA; a.nc = nB;
  a.K = ldz;
  a.symmetric = sym ? 1 : 0;
  a.vec_ok = 1;
  cudaError_t e;
  if (use == GT_EVERYTHING) {
    const int64_t t = cdiv(nA, 128) * cdiv(nB, 128) / (sym ? 2 : 1);
    if (t >= 2 * sm_count())
      e = launch_allpairs_simt<OpDot, OutPearsonF32, 8, 8>(a, OpDot{}, OutPearsonF32{po}, s);
    else
      e = launch_allpairs_simt<OpDot, OutPearsonF32, 4, 4>(a, OpDot{}, OutPearsonF32{po}, s);
  } else {
    e = launch_allpairs_simt<OpPairwise, OutPairwise, 4, 4>(a, OpPairwise{}, OutPairwise{po}, s);
  }
  if (e != cudaSuccess) return fail(GT_ECUDA, "pearson kernel launch: %s", cudaGetErrorString(e));
  return GT_OK;
}
