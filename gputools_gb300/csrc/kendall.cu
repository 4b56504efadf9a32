// kendall.cu -- gpuCor(method = "kendall"): tau-b from exact integer counts.
//
// Reference: src/kendall.cpp:13-55 masterKendall() launches
// inst/cuda/kendall.cu:4-47 gpuKendall, one 16x16 block per variable pair
// that loops over all observation pairs with float counters (exact only below
// 2^24) and reports (C - (T - C)) / T with joint ties counted as concordant,
// which is not R's cor(method = "kendall").
//
// Here the observation pairs are bit-sliced once per variable:
//   pair p = (i, (i + d) mod n), d = 1 .. floor(n/2), i = 0 .. n-1
//   (for even n the row d = n/2 keeps only i < n/2), which enumerates every
//   unordered pair exactly once in rows of n bits;
//   U_v[p] = x_v[j] != x_v[i]   (pair not tied),   G_v[p] = x_v[j] > x_v[i].
// For a variable pair (x, y), with m = U_x & U_y:
//   concordant - discordant = popc(m) - 2 popc(m & (G_x ^ G_y)),
// accumulated over 32-bit words by a shared-memory-tiled CUDA-core kernel
// (64x64 variable tiles, 128-bit loads, split over the pair dimension with
// 64-bit atomics).  Tx = popc(U_x).  tau-b = S / (sqrt(Tx) * sqrt(Ty)) is then
// evaluated in IEEE double with explicit round-to-nearest operations in R's
// order, clamped to [-1, 1]; NaN when either variable is constant; exactly 1
// on the diagonal of cor(x).
#include "common.cuh"
#include "kernels.cuh"

#include <cmath>

namespace gt {

namespace {

constexpr int kKT = 256;        // threads per count CTA
constexpr int kKBK = 16;        // words per shared slab
constexpr int kKLd = 18;        // padded shared row, in words (uint2)

// One warp per chunk of 32 consecutive words of one variable's rows d0+1 ..
// d0+drows (Wn words each): for word (d, w), lane b handles i = 32 w + b and
// the ballots form the word; lane e keeps word e of the chunk, so the chunk
// is stored with one coalesced 256-byte store, and the untied count goes to
// T[v] with one atomic per chunk.
__global__ void kendall_masks_kernel(const float *__restrict__ X, int64_t nvar, int64_t n,
                                     int64_t d0, int64_t drows, int64_t Wn,
                                     uint2 *__restrict__ M, unsigned long long *__restrict__ T) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int64_t per_var = drows * Wn, chunks = (per_var + 31) / 32;
  for (int64_t t = warp; t < nvar * chunks; t += nwarps) {
    const int64_t v = t / chunks, base = (t - v * chunks) * 32;
    const int cnt = per_var - base < 32 ? int(per_var - base) : 32;
    const float *x = X + v * n;
    int64_t dr = base / Wn, w = base - dr * Wn;
    uint2 mine = make_uint2(0u, 0u);
    unsigned long long untied_bits = 0;
    for (int e = 0; e < cnt; e++) {  // warp-uniform
      const int64_t d = d0 + dr + 1, i = 32 * w + lane;
      bool untied = false, greater = false;
      if (i < n && (2 * d < n || i < n / 2)) {
        int64_t j = i + d;
        if (j >= n) j -= n;
        const float xi = x[i], xj = x[j];
        untied = xj != xi;
        greater = xj > xi;
      }
      const unsigned u = __ballot_sync(0xffffffffu, untied);
      const unsigned g = __ballot_sync(0xffffffffu, greater);
      if (lane == e) mine = make_uint2(u, g);
      untied_bits += __popc(u);
      if (++w == Wn) {
        w = 0;
        dr++;
      }
    }
    if (lane < cnt) M[v * per_var + base + lane] = mine;
    if (lane == 0 && untied_bits) atomicAdd(&T[v], untied_bits);
  }
}

// The same words, chunks and untied counts from a variable's observations
// staged once in shared memory: one CTA per variable, for n up to
// kKmSmemN (every word otherwise reads both of its observations from L1/L2).
constexpr int kKmThreads = 256;
constexpr int64_t kKmSmemN = 12288;  // 48 KB of observations
__global__ void __launch_bounds__(kKmThreads)
kendall_masks_smem_kernel(const float *__restrict__ X, int n, int d0, int drows, int Wn,
                          uint2 *__restrict__ M, unsigned long long *__restrict__ T) {
  extern __shared__ float xs[];  // [n]
  __shared__ unsigned long long part[kKmThreads / 32];
  const int64_t v = blockIdx.x;
  const float *x = X + v * int64_t(n);
  for (int k = threadIdx.x; k < n; k += kKmThreads) xs[k] = x[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t per_var = int64_t(drows) * Wn;
  const int64_t chunks = (per_var + 31) / 32;
  unsigned long long untied_bits = 0;
  for (int64_t c = warp; c < chunks; c += kKmThreads / 32) {
    const int64_t base = c * 32;
    const int cnt = per_var - base < 32 ? int(per_var - base) : 32;
    int dr = int(base / Wn), w = int(base - int64_t(dr) * Wn);
    uint2 mine = make_uint2(0u, 0u);
    for (int e = 0; e < cnt; e++) {  // warp-uniform
      const int d = d0 + dr + 1, i = 32 * w + lane;
      bool untied = false, greater = false;
      if (i < n && (2 * d < n || i < n / 2)) {
        int j = i + d;
        if (j >= n) j -= n;
        const float xi = xs[i], xj = xs[j];
        untied = xj != xi;
        greater = xj > xi;
      }
      const unsigned u = __ballot_sync(0xffffffffu, untied);
      const unsigned g = __ballot_sync(0xffffffffu, greater);
      if (lane == e) mine = make_uint2(u, g);
      untied_bits += __popc(u);
      if (++w == Wn) {
        w = 0;
        dr++;
      }
    }
    if (lane < cnt) M[v * per_var + base + lane] = mine;
  }
  if (lane == 0) part[warp] = untied_bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int q = 0; q < kKmThreads / 32; q++) tot += part[q];
    if (tot) atomicAdd(&T[v], tot);
  }
}

// Counts of one 64 x 64 tile of variable pairs over words [kbeg, kend):
// both[i][j] = popc(m), disc[i][j] = popc(m & (Gr ^ Gc)) with m = Ur & Uc,
// for rows row0 + ty + 16 i of MR and columns col0 + tx + 16 j of MC.
__device__ __forceinline__ void tile_counts(const uint2 *__restrict__ MR, int64_t nr,
                                            const uint2 *__restrict__ MC, int64_t nc, int64_t K,
                                            int64_t row0, int64_t col0, int64_t kbeg,
                                            int64_t kend, uint2 *sR, uint2 *sC,
                                            unsigned (&both)[4][4], unsigned (&disc)[4][4]) {
  constexpr int TM = 4, TN = 4;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) both[i][j] = disc[i][j] = 0u;
  for (int64_t k0 = kbeg; k0 < kend; k0 += kKBK) {
    // 64 rows x 16 words = 512 uint4 (two words each) per operand.
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const int q = threadIdx.x + s * kKT;
      const int row = q >> 3, c2 = q & 7;
      const int64_t gk = k0 + 2 * c2;
      uint4 vr = make_uint4(0u, 0u, 0u, 0u), vc = make_uint4(0u, 0u, 0u, 0u);
      const int64_t gr = row0 + row, gc = col0 + row;
      if (gr < nr) {
        if (gk < kend) { const uint2 w = MR[gr * K + gk]; vr.x = w.x; vr.y = w.y; }
        if (gk + 1 < kend) { const uint2 w = MR[gr * K + gk + 1]; vr.z = w.x; vr.w = w.y; }
      }
      if (gc < nc) {
        if (gk < kend) { const uint2 w = MC[gc * K + gk]; vc.x = w.x; vc.y = w.y; }
        if (gk + 1 < kend) { const uint2 w = MC[gc * K + gk + 1]; vc.z = w.x; vc.w = w.y; }
      }
      *reinterpret_cast<uint4 *>(&sR[row * kKLd + 2 * c2]) = vr;
      *reinterpret_cast<uint4 *>(&sC[row * kKLd + 2 * c2]) = vc;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKBK / 2; kk++) {
      uint4 a[TM];
#pragma unroll
      for (int i = 0; i < TM; i++)
        a[i] = *reinterpret_cast<const uint4 *>(&sR[(ty + 16 * i) * kKLd + 2 * kk]);
#pragma unroll
      for (int j = 0; j < TN; j++) {
        const uint4 b = *reinterpret_cast<const uint4 *>(&sC[(tx + 16 * j) * kKLd + 2 * kk]);
#pragma unroll
        for (int i = 0; i < TM; i++) {
          const unsigned m0 = a[i].x & b.x, m1 = a[i].z & b.z;
          both[i][j] += __popc(m0) + __popc(m1);
          disc[i][j] += __popc(m0 & (a[i].y ^ b.y)) + __popc(m1 & (a[i].w ^ b.w));
        }
      }
    }
    __syncthreads();
  }
}

// tau-b = S / (sqrt(Tx) * sqrt(Ty)) in IEEE double, R's evaluation order,
// clamped to [-1, 1]; NaN when either variable is constant.  rx = sqrt(Tx)
// and ry = sqrt(Ty) (__dsqrt_rn) are taken once per variable.
__device__ __forceinline__ double taub(long long S, double rx, double ry) {
  if (rx == 0.0 || ry == 0.0) return __longlong_as_double(0x7ff8000000000000LL);
  double r = __ddiv_rn(double(S), __dmul_rn(rx, ry));
  if (r > 1.0) r = 1.0;
  if (r < -1.0) r = -1.0;
  return r;
}

// S[r*ld + c] += sum over words of popc(m) - 2 popc(m & (Gr ^ Gc)).
// Rows r index MR (the Y set), columns c index MC (the X set).
__global__ void __launch_bounds__(kKT)
kendall_count_kernel(const uint2 *__restrict__ MR, int64_t nr, const uint2 *__restrict__ MC,
                     int64_t nc, int64_t K, int64_t kchunk, int symmetric,
                     unsigned long long *__restrict__ S, int64_t ld) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (symmetric && ti > tj) return;
  const int64_t row0 = int64_t(ti) * 64, col0 = int64_t(tj) * 64;
  const int64_t kbeg = int64_t(blockIdx.z) * kchunk;
  const int64_t kend = min(K, kbeg + kchunk);
  if (kbeg >= kend) return;
  __shared__ __align__(16) uint2 sR[64 * kKLd];
  __shared__ __align__(16) uint2 sC[64 * kKLd];
  unsigned both[4][4], disc[4][4];
  tile_counts(MR, nr, MC, nc, K, row0, col0, kbeg, kend, sR, sC, both, disc);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const bool mirror = symmetric && ti != tj;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int64_t r = row0 + ty + 16 * i;
    if (r >= nr) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int64_t c = col0 + tx + 16 * j;
      if (c >= nc) continue;
      const long long sv = (long long)both[i][j] - 2LL * (long long)disc[i][j];
      atomicAdd(&S[r * ld + c], (unsigned long long)sv);
      if (mirror) atomicAdd(&S[c * ld + r], (unsigned long long)sv);
    }
  }
}

// sqrt(T_v) of every variable, the factors of tau-b's denominator.
__global__ void kendall_roots_kernel(const unsigned long long *__restrict__ T, int64_t nvar,
                                     double *__restrict__ root) {
  const int64_t v = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (v < nvar) root[v] = __dsqrt_rn(double(T[v]));
}

// out[y*nx + x] = tau-b; a block walks whole rows, so no index is divided.
__global__ void kendall_finish_kernel(const unsigned long long *__restrict__ S,
                                      const double *__restrict__ RX,
                                      const double *__restrict__ RY, int64_t nx, int64_t ny,
                                      int same, double *__restrict__ out) {
  for (int64_t y = blockIdx.x; y < ny; y += gridDim.x) {
    const double ry = RY[y];
    for (int64_t x = threadIdx.x; x < nx; x += blockDim.x) {
      const int64_t i = y * nx + x;
      out[i] = (same && x == y) ? 1.0 : taub((long long)S[i], RX[x], ry);
    }
  }
}

int grid_cap(int64_t work, int threads) {
  const int64_t g = cdiv(work, threads);
  const int64_t cap = int64_t(sm_count()) * 16;
  return int(g < 1 ? 1 : (g > cap ? cap : g));
}

// The masks of pair rows d0 + 1 .. d0 + dr of nv variables (and their untied
// counts added to T): observations staged in shared memory when they fit.
void launch_kendall_masks(const float *X, int64_t nv, int64_t n, int64_t d0, int64_t dr,
                          int64_t Wn, uint2 *M, unsigned long long *T, cudaStream_t s) {
  if (n <= kKmSmemN && nv <= 2147483647LL) {
    kendall_masks_smem_kernel<<<unsigned(nv), kKmThreads, size_t(n) * sizeof(float), s>>>(
        X, int(n), int(d0), int(dr), int(Wn), M, T);
  } else {
    kendall_masks_kernel<<<grid_cap(nv * cdiv(dr * Wn, 32) * 32, 256), 256, 0, s>>>(X, nv, n, d0,
                                                                                  dr, Wn, M, T);
  }
  count_launch();
}

}  // namespace

int kendall_impl(const float *dX, int64_t nx, const float *dY, int64_t ny, int64_t n, int same,
                 double *d_out, cudaStream_t s) {
  if (nx == 0 || ny == 0) return GT_OK;
  const int64_t Dr = n / 2;            // pair rows
  const int64_t Wn = cdiv(n, 32);      // words per pair row
  const int64_t nvar = same ? nx : nx + ny;
  // Mask memory per pair row for all variables; chunk the rows to a budget.
  const int64_t per_row = nvar * Wn * 8;
  const int64_t budget = int64_t(2) << 30;
  int64_t rows_chunk = per_row > 0 ? budget / per_row : Dr;
  if (rows_chunk < 1) rows_chunk = 1;
  if (rows_chunk > Dr) rows_chunk = Dr;

  void *pS = nullptr, *pT = nullptr, *pM = nullptr;
  GT_TRY(ws_get(WS_SCRATCH0, size_t(nx) * size_t(ny) * 8, &pS));
  GT_TRY(ws_get(WS_SCRATCH1, size_t(nvar) * 16, &pT));  // untied counts, then their roots
  auto *S = static_cast<unsigned long long *>(pS);
  auto *T = static_cast<unsigned long long *>(pT);
  auto *root = reinterpret_cast<double *>(T + nvar);
  GT_CUDA(cudaMemsetAsync(S, 0, size_t(nx) * size_t(ny) * 8, s));
  GT_CUDA(cudaMemsetAsync(T, 0, size_t(nvar) * 8, s));
  unsigned long long *TX = T, *TY = same ? T : T + nx;

  if (Dr > 0) {
    GT_TRY(ws_get(WS_SCRATCH2, size_t(nvar) * size_t(rows_chunk) * size_t(Wn) * 8, &pM));
    uint2 *M = static_cast<uint2 *>(pM);
    for (int64_t d0 = 0; d0 < Dr; d0 += rows_chunk) {
      const int64_t dr = (Dr - d0 < rows_chunk) ? Dr - d0 : rows_chunk;
      const int64_t K = dr * Wn;
      uint2 *MXs = M, *MYs = same ? M : M + nx * K;
      launch_kendall_masks(dX, nx, n, d0, dr, Wn, MXs, TX, s);
      if (!same) launch_kendall_masks(dY, ny, n, d0, dr, Wn, MYs, TY, s);
      const int64_t gy = cdiv(ny, 64), gx = cdiv(nx, 64);
      if (gy > 65535 || gx > 2147483647LL) return fail(GT_EINVAL, "too many variables");
      const int64_t tiles = same ? gx * (gx + 1) / 2 : gx * gy;
      int64_t splits = cdiv(2 * sm_count(), tiles);
      const int64_t max_splits = cdiv(K, 256);
      if (splits > max_splits) splits = max_splits;
      if (splits < 1) splits = 1;
      if (splits > 65535) splits = 65535;
      const int64_t kchunk = cdiv(cdiv(K, splits), kKBK) * kKBK;
      splits = cdiv(K, kchunk);
      dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)splits);
      ProfScope prof("kendall_count", s);
      kendall_count_kernel<<<grid, kKT, 0, s>>>(MYs, ny, MXs, nx, K, kchunk, same, S, nx);
      count_launch();
      GT_CUDA(cudaGetLastError());
    }
  }
  kendall_roots_kernel<<<unsigned(cdiv(nvar, 256)), 256, 0, s>>>(T, nvar, root);
  const double *RX = root, *RY = same ? root : root + nx;
  const int64_t fgrid = ny < int64_t(sm_count()) * 16 ? ny : int64_t(sm_count()) * 16;
  kendall_finish_kernel<<<unsigned(fgrid), 256, 0, s>>>(S, RX, RY, nx, ny, same, d_out);
  count_launch(2);
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

// ---------------------------------------------------------------- batches
// Many independent Kendall problems in one pass: one CTA per variable builds
// its pair masks and untied count; one count launch walks per-CTA lists of
// 64 x 64 tiles (balanced on the host) across all problems and writes tau-b
// directly (each tile covers its problem's full pair dimension).

namespace {

__device__ __forceinline__ int64_t find_segment(const int64_t *__restrict__ prefix, int64_t n,
                                                int64_t x) {
  int64_t lo = 0, hi = n;  // prefix has n + 1 entries; largest i with prefix[i] <= x
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (prefix[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

constexpr int kKbMaskThreads = 128;
constexpr int kKbStage = 4096;  // observations staged in shared memory (16 KB)

// One CTA per variable of the batch: warps take chunks of 32 consecutive
// words (lane e keeps word e, one coalesced store per chunk), reading the
// observations from shared memory when they fit; the untied count is the
// CTA's sum.  The same words and counts either way.
__global__ void __launch_bounds__(kKbMaskThreads)
kendall_batch_masks_kernel(const KendallBatchProblem *__restrict__ P,
                           const int64_t *__restrict__ var_prefix, int64_t nprob,
                           uint2 *__restrict__ M, unsigned long long *__restrict__ T,
                           double *__restrict__ root) {
  __shared__ unsigned long long part[kKbMaskThreads / 32];
  __shared__ float xs[kKbStage];
  const int64_t gv = blockIdx.x;
  const int64_t pi = find_segment(var_prefix, nprob, gv);
  const KendallBatchProblem pr = P[pi];
  const int64_t v = gv - var_prefix[pi];
  const float *x = pr.X + v * pr.n;
  uint2 *mv = M + pr.mask_off + v * pr.K;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool staged = pr.n <= kKbStage;  // CTA-uniform
  if (staged) {
    for (int64_t k = threadIdx.x; k < pr.n; k += kKbMaskThreads) xs[k] = x[k];
    __syncthreads();
  }
  const int64_t n = pr.n, Wn = pr.Wn, K = pr.K;
  unsigned long long cnt = 0;
  auto words = [&](auto rd) {
    for (int64_t base = 32 * int64_t(warp); base < K; base += 32 * (kKbMaskThreads / 32)) {
      const int m = K - base < 32 ? int(K - base) : 32;
      int64_t dr = base / Wn, w = base - dr * Wn;
      uint2 mine = make_uint2(0u, 0u);
      for (int e = 0; e < m; e++) {  // warp-uniform
        const int64_t d = dr + 1, i = 32 * w + lane;
        bool untied = false, greater = false;
        if (i < n && (2 * d < n || i < n / 2)) {
          int64_t j = i + d;
          if (j >= n) j -= n;
          const float xi = rd(i), xj = rd(j);
          untied = xj != xi;
          greater = xj > xi;
        }
        const unsigned u = __ballot_sync(0xffffffffu, untied);
        const unsigned g = __ballot_sync(0xffffffffu, greater);
        if (lane == e) mine = make_uint2(u, g);
        cnt += __popc(u);
        if (++w == Wn) {
          w = 0;
          dr++;
        }
      }
      if (lane < m) mv[base + lane] = mine;
    }
  };
  if (staged) words([&](int64_t k) { return xs[k]; });
  else words([&](int64_t k) { return x[k]; });
  if (lane == 0) part[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int q = 0; q < kKbMaskThreads / 32; q++) tot += part[q];
    T[pr.var_off + v] = tot;
    root[pr.var_off + v] = __dsqrt_rn(double(tot));
  }
}

__global__ void __launch_bounds__(kKT)
kendall_batch_count_kernel(const KendallBatchProblem *__restrict__ P,
                           const int64_t *__restrict__ tile_prefix, int64_t nprob,
                           const int64_t *__restrict__ cta_tiles,
                           const int64_t *__restrict__ cta_off, const uint2 *__restrict__ M,
                           const double *__restrict__ root) {
  __shared__ __align__(16) uint2 sR[64 * kKLd];
  __shared__ __align__(16) uint2 sC[64 * kKLd];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int64_t idx = cta_off[blockIdx.x]; idx < cta_off[blockIdx.x + 1]; idx++) {
    const int64_t gtile = cta_tiles[idx];
    const int64_t pi = find_segment(tile_prefix, nprob, gtile);
    const KendallBatchProblem pr = P[pi];
    const int64_t lt = gtile - tile_prefix[pi];
    int64_t tj = int64_t((sqrt(8.0 * double(lt) + 1.0) - 1.0) * 0.5);
    while ((tj + 1) * (tj + 2) / 2 <= lt) tj++;
    while (tj * (tj + 1) / 2 > lt) tj--;
    const int64_t ti = lt - tj * (tj + 1) / 2;  // ti <= tj
    const uint2 *Mp = M + pr.mask_off;
    unsigned both[4][4], disc[4][4];
    const int64_t row0 = ti * 64, col0 = tj * 64;
    tile_counts(Mp, pr.p, Mp, pr.p, pr.K, row0, col0, 0, pr.K, sR, sC, both, disc);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int64_t r = row0 + ty + 16 * i;
      if (r >= pr.p) continue;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int64_t c = col0 + tx + 16 * j;
        if (c >= pr.p) continue;
        const long long sv = (long long)both[i][j] - 2LL * (long long)disc[i][j];
        const double tau =
            (r == c) ? 1.0 : taub(sv, root[pr.var_off + c], root[pr.var_off + r]);
        pr.out[r * pr.p + c] = tau;
        if (ti != tj) pr.out[c * pr.p + r] = tau;
      }
    }
  }
}

}  // namespace

int kendall_batch_launch(const KendallBatchProblem *d_probs, const int64_t *d_var_prefix,
                         int64_t nprob, int64_t total_vars, const int64_t *d_tile_prefix,
                         const int64_t *d_cta_tiles, const int64_t *d_cta_off, int64_t ncta,
                         uint2 *d_masks, unsigned long long *d_T, cudaStream_t s) {
  // d_T holds the untied counts of all variables, then their square roots
  double *root = reinterpret_cast<double *>(d_T + total_vars);
  if (total_vars > 0) {
    kendall_batch_masks_kernel<<<unsigned(total_vars), kKbMaskThreads, 0, s>>>(
        d_probs, d_var_prefix, nprob, d_masks, d_T, root);
    count_launch();
  }
  if (ncta > 0) {
    kendall_batch_count_kernel<<<unsigned(ncta), kKT, 0, s>>>(d_probs, d_tile_prefix, nprob,
                                                             d_cta_tiles, d_cta_off, d_masks, root);
    count_launch();
  }
  GT_CUDA(cudaGetLastError());
  return GT_OK;
}

int kendall_check(int64_t nx, int64_t ny, int64_t n) {
  if (nx < 0 || ny < 0 || n < 0) return fail(GT_EINVAL, "negative size");
  if (n > 65536) return fail(GT_EINVAL, "kendall supports at most 65536 observations (n=%lld)",
                             (long long)n);
  return GT_OK;
}

int same_contents(const float *a, const float *b, int64_t count, bool *same, cudaStream_t s);

}  // namespace gt

extern "C" int gt_kendall_device(const float *d_X, int64_t nx, const float *d_Y, int64_t ny,
                                 int64_t n, double *d_out, void *stream) {
  gt::clear_error();
  GT_TRY(gt::kendall_check(nx, ny, n));
  if ((nx > 0 && !d_X) || (ny > 0 && !d_Y) || (nx * ny > 0 && !d_out))
    return gt::fail(GT_EINVAL, "null device pointer");
  const int same = (d_X == d_Y && nx == ny) ? 1 : 0;
  return gt::kendall_impl(d_X, nx, d_Y, ny, n, same, d_out, static_cast<cudaStream_t>(stream));
}

extern "C" int gt_kendall(const float *X, int64_t nx, const float *Y, int64_t ny, int64_t n,
                          double *out) {
  gt::clear_error();
  GT_TRY(gt::kendall_check(nx, ny, n));
  if (nx == 0 || ny == 0) return GT_OK;
  if (!X || !Y || !out) return gt::fail(GT_EINVAL, "null host pointer");
  cudaStream_t s = gt::lib_stream();
  gt::StreamSyncGuard guard(s);
  const size_t bx = size_t(nx) * size_t(n) * 4, by = size_t(ny) * size_t(n) * 4;
  void *dX = nullptr, *dY = nullptr, *dO = nullptr;
  GT_TRY(gt::ws_get(gt::WS_IN_A, bx, &dX));
  GT_CUDA(cudaMemcpyAsync(dX, X, bx, cudaMemcpyHostToDevice, s));
  bool same = (X == Y && nx == ny);
  if (!same) {
    GT_TRY(gt::ws_get(gt::WS_IN_B, by, &dY));
    GT_CUDA(cudaMemcpyAsync(dY, Y, by, cudaMemcpyHostToDevice, s));
    if (nx == ny)
      GT_TRY(gt::same_contents(static_cast<float *>(dX), static_cast<float *>(dY), nx * n, &same, s));
  }
  if (same) dY = dX;
  void *direct = gt::host_output_ptr(out, size_t(nx) * size_t(ny) * 8);
  if (!(dO = direct)) GT_TRY(gt::ws_get(gt::WS_OUT0, size_t(nx) * size_t(ny) * 8, &dO));
  GT_TRY(gt::kendall_impl(static_cast<float *>(dX), nx, static_cast<float *>(dY), ny, n,
                          same ? 1 : 0, static_cast<double *>(dO), s));
  if (!direct)
    GT_CUDA(cudaMemcpyAsync(out, dO, size_t(nx) * size_t(ny) * 8, cudaMemcpyDeviceToHost, s));
  GT_CUDA(cudaStreamSynchronize(s));
  return GT_OK;
}
