// distance.cu -- gpuDist's six metrics on CUDA cores.
//
// Reference: src/distance.cpp:209-316 (distance, distance_device) launching
// the `*_kernel_same` kernels of inst/cuda/distance.cu (euclidean :40-78,
// maximum :116-154, manhattan :192-232, canberra :273-316, binary :366-415,
// minkowski :453-493).  Those kernels use one 32-thread block per (x, y) with
// a shared-memory tree reduction; here every metric runs on the tiled engine
// of allpairs_simt.cuh, computing each unordered pair once.
//
// Semantics follow R's stats::dist (the reference's documented model):
//  * canberra omits terms whose numerator and denominator are both zero
//    (a = b = 0) and scales the sum by dim / terms-used; a term with a zero
//    denominator only (a = -b != 0) is +Inf.  The reference kernel instead
//    skips every zero-denominator term and never rescales
//    (inst/cuda/distance.cu:294), so the two differ only when zeros occur.
//  * minkowski evaluates |a-b|^p exactly for p = 1, 2, 3 and as
//    2^(p log2 |a-b|) otherwise (the reference uses the low-accuracy __powf,
//    :471, :487); the final root is FP32 (cbrtf for p = 3, else 2^(log2(s) / p)).
#include "common.cuh"
#include "allpairs_simt.cuh"
#include "kernels.cuh"

#include <cmath>

namespace gt {

namespace {

struct OpEuclid {
  static constexpr int kUnrollK = 1;  // measured fastest (up to 10 % over a full unroll)
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const {
    const float d = a - b;
    c[0] = fmaf(d, d, c[0]);
  }
  __device__ float finish(const float (&c)[1], int64_t) const { return sqrtf(c[0]); }
};

struct OpManhattan {
  static constexpr int kUnrollK = 1;  // measured fastest (up to 10 % over a full unroll)
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const { c[0] += fabsf(a - b); }
  __device__ float finish(const float (&c)[1], int64_t) const { return c[0]; }
};

struct OpMaximum {
  static constexpr int kUnrollK = 1;  // measured fastest (up to 10 % over a full unroll)
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const { c[0] = fmaxf(c[0], fabsf(a - b)); }
  __device__ float finish(const float (&c)[1], int64_t) const { return c[0]; }
};

struct OpCanberra {
  static constexpr int kUnrollK = 4;  // fully unrolled divisions: 16 % slower
  static constexpr int NACC = 2;  // sum of terms, number of terms used
  static constexpr bool kSkipPad = true;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[2]) const { c[0] = 0.f; c[1] = 0.f; }
  __device__ void step(float (&c)[2], float a, float b) const {
    const bool used = (a != 0.f) | (b != 0.f);
    const float t = __fdiv_rn(fabsf(a - b), fabsf(a + b));
    c[0] += used ? t : 0.f;
    c[1] += used ? 1.f : 0.f;
  }
  __device__ float finish(const float (&c)[2], int64_t K) const {
    if (c[1] == 0.f) return __int_as_float(0x7fc00000);
    if (double(c[1]) < double(K)) return float(double(c[0]) / (double(c[1]) / double(K)));
    return c[0];
  }
};

// Binary on bit-packed points (bit k of word w: coordinate 32 w + k is
// nonzero); the engine carries the words as float bit patterns and the two
// counts (bits on in exactly one point, bits on in either) as integers in
// the accumulator slots.  The reference counts per coordinate in float
// (inst/cuda/distance.cu:366-415); the counts, and so the results, are the same.
struct OpBinaryBits {
  static constexpr int NACC = 2;  // bits on in exactly one, bits on in either
  static constexpr bool kSkipPad = true;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[2]) const { c[0] = __int_as_float(0); c[1] = __int_as_float(0); }
  __device__ void step(float (&c)[2], float a, float b) const {
    const unsigned x = __float_as_uint(a), y = __float_as_uint(b);
    c[0] = __int_as_float(__float_as_int(c[0]) + __popc(x ^ y));
    c[1] = __int_as_float(__float_as_int(c[1]) + __popc(x | y));
  }
  __device__ float finish(const float (&c)[2], int64_t) const {
    const float d = float(__float_as_int(c[1]));
    return d != 0.f ? float(__float_as_int(c[0])) / d : 0.f;
  }
};

// The same counts packed in one 32-bit accumulator (bits on in either << 16 |
// bits on in exactly one), for fewer than 65536 coordinates, where neither
// count can carry out of its half: a single-accumulator operation, so large
// problems take the 128 x 128 tiles (the binary kernel spends its time per
// tile, not on its two words of arithmetic per pair).
struct OpBinaryPacked {
  static constexpr int NACC = 1;
  static constexpr bool kSkipPad = true;
  static constexpr int kUnrollK = 1;  // a few words per point: the slab's loop stops early
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = __uint_as_float(0u); }
  __device__ void step(float (&c)[1], float a, float b) const {
    const unsigned x = __float_as_uint(a), y = __float_as_uint(b);
    c[0] = __uint_as_float(__float_as_uint(c[0]) + __popc(x ^ y) +
                           (unsigned(__popc(x | y)) << 16));
  }
  __device__ float finish(const float (&c)[1], int64_t) const {
    const unsigned v = __float_as_uint(c[0]);
    const float d = float(int(v >> 16));
    return d != 0.f ? float(int(v & 0xffffu)) / d : 0.f;
  }
};

// One warp per point: word w of point i holds the nonzero pattern of
// coordinates 32 w .. 32 w + 31 (NaN counts as nonzero, as in OpBinary).
__global__ void __launch_bounds__(256)
pack_nonzero_kernel(const float *__restrict__ P, int64_t n, int64_t dim, int64_t words,
                    unsigned *__restrict__ bits) {
  const int64_t i = (int64_t(blockIdx.x) * 256 + threadIdx.x) >> 5;
  if (i >= n) return;  // whole warps
  const int lane = threadIdx.x & 31;
  for (int64_t w = 0; w < words; w++) {
    const int64_t k = 32 * w + lane;
    const unsigned b = __ballot_sync(0xffffffffu, k < dim && P[i * dim + k] != 0.f);
    if (lane == 0) bits[i * words + w] = b;
  }
}

struct OpMink3 {
  static constexpr int kUnrollK = 1;  // measured fastest (up to 10 % over a full unroll)
  static constexpr int NACC = 1;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  __device__ void step(float (&c)[1], float a, float b) const {
    const float d = fabsf(a - b);
    c[0] = fmaf(d * d, d, c[0]);
  }
  // FP32 root: one FP64 root per entry would cost GB300 more than the entry's
  // whole sum (its FP64 rate is ~1/64 of FP32); cbrtf is within 1 ulp
  __device__ float finish(const float (&c)[1], int64_t) const { return cbrtf(c[0]); }
};

struct OpMinkP {
  static constexpr int kUnrollK = 1;  // measured fastest (up to 10 % over a full unroll)
  static constexpr int NACC = 1;
  float p;
  __device__ static float pad() { return 0.f; }
  __device__ void init(float (&c)[1]) const { c[0] = 0.f; }
  // |a - b|^p as 2^(p log2 |a - b|) (0, Inf and NaN come out as from powf;
  // relative error about 2 |p log2 |a - b|| ulp, against powf's 1 ulp, at less
  // than half of powf's instructions)
  __device__ void step(float (&c)[1], float a, float b) const {
    c[0] += exp2f(p * log2f(fabsf(a - b)));
  }
  // s^(1/p) in FP32 as 2^(log2(s) / p): relative error about |log2 s| ulp
  __device__ float finish(const float (&c)[1], int64_t) const {
    return c[0] > 0.f ? exp2f(__fdiv_rn(log2f(c[0]), p)) : c[0];
  }
};

// Writes one distance in the full square layout (d[y*n + x], both halves)
// or R's dist layout (strict lower triangle by columns).
template <class Op>
struct OutDist {
  Op op;
  float *out;
  int64_t n, K;
  int layout;
  // the full layout's mirror goes through shared memory (coalesced stores)
  static constexpr bool kStagedMirror = true;
  __device__ bool staged(bool mirror) const { return mirror && layout == GT_LAYOUT_FULL; }
  __device__ float value(int64_t r, int64_t c, const float (&acc)[Op::NACC]) const {
    return (r == c) ? 0.f : op.finish(acc, K);
  }
  __device__ void store(int64_t r, int64_t c, float v) const { out[r * n + c] = v; }
  __device__ void operator()(int64_t r, int64_t c, const float (&acc)[Op::NACC], bool mirror) const {
    if (layout == GT_LAYOUT_FULL) {
      const float v = (r == c) ? 0.f : op.finish(acc, K);
      out[r * n + c] = v;
      if (mirror) out[c * n + r] = v;
    } else {
      if (c <= r) return;  // each unordered pair once; (r, c) with c > r
      const int64_t i = c, j = r;
      out[n * j - j * (j + 1) / 2 + i - j - 1] = op.finish(acc, K);
    }
  }
};

template <class Op>
cudaError_t run_metric(const Op &op, const float *pts, int64_t n, int64_t dim, float *out,
                       int layout, cudaStream_t st) {
  SimtArgs a;
  a.R = a.C = pts;
  a.ldr = a.ldc = dim;
  a.nr = a.nc = n;
  a.K = dim;
  a.symmetric = 1;
  a.vec_ok = (dim % 4 == 0) && aligned16(pts);
  OutDist<Op> o{op, out, n, dim, layout};
  ProfScope prof("dist", st);
  const int64_t t128 = cdiv(n, 128);
  if (Op::NACC == 1 && t128 * (t128 + 1) / 2 >= 2 * sm_count())
    return launch_allpairs_simt<Op, OutDist<Op>, 8, 8>(a, op, o, st);
  return launch_allpairs_simt<Op, OutDist<Op>, 4, 4>(a, op, o, st);
}

}  // namespace

int dist_check_args(int64_t n, int64_t dim, int method, int layout) {
  if (n < 0 || dim < 0) return fail(GT_EINVAL, "negative size (n=%lld, dim=%lld)",
                                    (long long)n, (long long)dim);
  if (method < GT_EUCLIDEAN || method > GT_MINKOWSKI)
    return fail(GT_EINVAL, "unknown distance method %d", method);
  if (layout != GT_LAYOUT_FULL && layout != GT_LAYOUT_DIST)
    return fail(GT_EINVAL, "unknown output layout %d", layout);
  if (cdiv(n, 64) > 65535) return fail(GT_EINVAL, "too many points (%lld)", (long long)n);
  return GT_OK;
}

// Euclidean distances on the FP32 CUDA-core path; used directly for
// GT_GRAM_FP32 and as the reference point of the tensor-core path.
int dist_simt(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout, int method,
              float p, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  switch (method) {
  case GT_EUCLIDEAN: e = run_metric(OpEuclid{}, d_pts, n, dim, d_out, layout, st); break;
  case GT_MAXIMUM: e = run_metric(OpMaximum{}, d_pts, n, dim, d_out, layout, st); break;
  case GT_MANHATTAN: e = run_metric(OpManhattan{}, d_pts, n, dim, d_out, layout, st); break;
  case GT_CANBERRA: e = run_metric(OpCanberra{}, d_pts, n, dim, d_out, layout, st); break;
  case GT_BINARY: {
    const int64_t words = cdiv(dim, 32);
    void *pb = nullptr;
    GT_TRY(ws_get(WS_SCRATCH0, size_t(n) * size_t(words) * 4, &pb));
    pack_nonzero_kernel<<<unsigned(cdiv(n, 8)), 256, 0, st>>>(d_pts, n, dim, words,
                                                             static_cast<unsigned *>(pb));
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess) {
      const float *bits = static_cast<const float *>(pb);
      e = dim < 65536 ? run_metric(OpBinaryPacked{}, bits, n, words, d_out, layout, st)
                      : run_metric(OpBinaryBits{}, bits, n, words, d_out, layout, st);
    }
    break;
  }
  case GT_MINKOWSKI:
    if (p == 1.f) e = run_metric(OpManhattan{}, d_pts, n, dim, d_out, layout, st);
    else if (p == 2.f) e = run_metric(OpEuclid{}, d_pts, n, dim, d_out, layout, st);
    else if (p == 3.f) e = run_metric(OpMink3{}, d_pts, n, dim, d_out, layout, st);
    else e = run_metric(OpMinkP{p}, d_pts, n, dim, d_out, layout, st);
    break;
  default: return fail(GT_EINVAL, "unknown distance method %d", method);
  }
  if (e != cudaSuccess) return fail(GT_ECUDA, "distance kernel launch: %s", cudaGetErrorString(e));
  return GT_OK;
}

}  // namespace gt

extern "C" int gt_distances_device(const float *d_points, int64_t n, int64_t dim, float *d_out,
                                   int layout, int method, float p, void *stream) {
  gt::clear_error();
  GT_TRY(gt::dist_check_args(n, dim, method, layout));
  if (n == 0) return GT_OK;
  if (!d_points || !d_out) return gt::fail(GT_EINVAL, "null device pointer");
  if (method == GT_MINKOWSKI && !(p > 0.f))
    return gt::fail(GT_EINVAL, "minkowski power must be positive (p=%g)", double(p));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (method == GT_EUCLIDEAN && gt_get_gram_path() != GT_GRAM_FP32)
    return gt::euclid_tc(d_points, n, dim, d_out, layout, st);
  return gt::dist_simt(d_points, n, dim, d_out, layout, method, p, st);
}

extern "C" int gt_distances(const float *points, int64_t n, int64_t dim, float *out, int method,
                            float p) {
  gt::clear_error();
  GT_TRY(gt::dist_check_args(n, dim, method, GT_LAYOUT_FULL));
  if (n == 0) return GT_OK;
  if (!points || !out) return gt::fail(GT_EINVAL, "null host pointer");
  cudaStream_t st = gt::lib_stream();
  gt::StreamSyncGuard guard(st);
  void *dp = nullptr, *dout = nullptr;
  GT_TRY(gt::ws_get(gt::WS_IN_A, size_t(n) * size_t(dim) * 4, &dp));
  void *direct = gt::host_output_ptr(out, size_t(n) * size_t(n) * 4);
  if (!(dout = direct)) GT_TRY(gt::ws_get(gt::WS_OUT0, size_t(n) * size_t(n) * 4, &dout));
  GT_CUDA(cudaMemcpyAsync(dp, points, size_t(n) * size_t(dim) * 4, cudaMemcpyHostToDevice, st));
  GT_TRY(gt_distances_device(static_cast<float *>(dp), n, dim, static_cast<float *>(dout),
                             GT_LAYOUT_FULL, method, p, st));
  if (!direct)
    GT_CUDA(cudaMemcpyAsync(out, dout, size_t(n) * size_t(n) * 4, cudaMemcpyDeviceToHost, st));
  GT_CUDA(cudaStreamSynchronize(st));
  bool failed = false;
  GT_TRY(gt::device_error_check(st, &failed));
  if (failed) return gt::fail(GT_ETIMEOUT, "a tensor-core kernel wait timed out");
  return GT_OK;
}
