// kernels.cuh -- internal entry points shared between the translation units
// of libgputools_gb300 (not part of the C ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <functional>
#include <vector>

#include "gputools_gb300.h"

namespace gt {

// distance.cu
int dist_check_args(int64_t n, int64_t dim, int method, int layout);
int dist_simt(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout, int method,
              float p, cudaStream_t st);

// gram_tc.cu: Euclidean distances as a split tcgen05 Gram contraction (f16x3
// when the Gram path is f16x3, else bf16x6) with compensated norms and an
// exact recomputation of near-zero distances.
int euclid_tc(const float *d_pts, int64_t n, int64_t dim, float *d_out, int layout,
              cudaStream_t st);

// gram_tc.cu: a 3-D TMA map over planes [nplanes][rows][kpad] of 16-bit
// values (box {bk, box_rows, 1}; bk 32 -> 64-byte swizzle, 64 -> 128-byte).
int tc_plane_map(CUtensorMap *map, const void *base, int64_t rows, int64_t kpad, int nplanes,
                 int box_rows, int bk, bool f16);

// Per-variable statistics of the Pearson prologue.
struct ColStats {
  double mean;
  double inv_norm;  // 1 / sqrt(sum (x - mean)^2), or 0 for a constant variable
  int flags;        // bit 0: contains NaN; bit 1: zero variance
};

int launch_colstats(const float *dX, int64_t nvar, int64_t n, int use, ColStats *st,
                    cudaStream_t s);

// gram_tc.cu: C[r][c] = sum_k Z_r[k] * Z_c[k] for the normalised Pearson
// operands on tcgen05 tensor cores, with the Pearson epilogue fused.
struct PearsonOut {
  float *corr, *ts, *pairs;
  int64_t ld;       // leading dimension of the outputs (nB)
  float npairs;     // value of `pairs` (everything mode: n)
  int symmetric;
  const int *gate = nullptr;  // tensor-core path: run only if *gate == 0 (device flag)
};

// Operands for the tensor-core path: for each variable, the 16-bit parts of
// split `kind` (enum gt_gram_path, not GT_GRAM_FP32) in planes of length kpad
// (multiple of 64), zero padded.
int pearson_tc(const void *d_zA, int64_t nA, const void *d_zB, int64_t nB, int64_t kpad,
               int kind, const PearsonOut &out, cudaStream_t st);

// gram_exact.cu: the error-free Pearson Gram (GT_GRAM_TC_F16X6): the
// prologue writes three fixed-point fp16 digit planes per variable
// ([plane][variable][kpad], kpad a multiple of 64), the Gram sums their
// products exactly in three TMEM accumulators, fused Pearson epilogue.
int pearson_exact_prologue(const float *dX, int64_t nvar, int64_t n, int slot_z, void **Z,
                           int64_t *kpad, cudaStream_t s);
int pearson_exact(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                  const PearsonOut &out, cudaStream_t s);
// The Pearson Gram on a device table of tiles (row0, col0) of 128 x 256 (see
// band_tiles in gram_core.cuh): f16x3 and f16x6; others GT_EUNSUPPORTED.
int pearson_tc_band(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad, int kind,
                    const PearsonOut &out, const int2 *tiles, int64_t ntiles, cudaStream_t s);
// band_tiles for callers outside the Gram sources: the tile table of a
// Pearson problem in bands of `band_blocks` row blocks of kGramRows rows.
constexpr int kGramRows = 128;
void pearson_band_tiles(int64_t nr, int64_t nc, bool symmetric, int64_t band_blocks,
                        std::vector<int2> &tiles, std::vector<int64_t> &offsets);
int pearson_exact_band(const void *zA, int64_t nA, const void *zB, int64_t nB, int64_t kpad,
                       const PearsonOut &out, const int2 *tiles, int64_t ntiles, cudaStream_t s);

// pairwise_tc.cu: pairwise-complete Pearson on the tensor cores (masked
// Gram of the six sums); every launch gated on the device flag run_if.
int pearson_pairwise_tc(const float *dA, int64_t nA, const float *dB, int64_t nB, int64_t n,
                        const PearsonOut &out, const int *run_if, cudaStream_t s);

// gram_tc.cu: B-spline mutual information from f16x3 weight planes ([part]
// [variable * 2^lg + bin][kpad], weights times 2^14, zero padded), entropies
// hx, hy; out[y * nx + x] (symmetric: X == Y, both triangles written).
int mi_tc(const void *planesX, int64_t rowsX, const void *planesY, int64_t rowsY, int64_t kpad,
          int lg, int nbins, int64_t nx, int64_t ny, int64_t nsamples, const float *hx,
          const float *hy, float *out, int symmetric, cudaStream_t s);

// C[r][c] = sum_k A_r[k] B_c[k] on tcgen05 from `nsplit` (2 or 3) split-bf16
// planes ([part][row][kpad], kpad a multiple of 64), stored as row-major float.
int gemm_tc_store(const void *planesA, int64_t nA, const void *planesB, int64_t nB, int64_t kpad,
                  int nsplit, float *C, int64_t ldc, cudaStream_t s);
// The bf16x6 contraction with its K range in up to `parts` (<= 4) pieces, one
// launch; piece q is stored into C + q * nA * ldc (*used pieces) and the
// caller adds them.
int gemm_tc_store_ksplit(const void *planesA, int64_t nA, const void *planesB, int64_t nB,
                         int64_t kpad, int parts, int *used, float *C, int64_t ldc,
                         cudaStream_t s);
// The same from f16x3 planes of rows scaled by powers of two; rsA / rsB hold
// the factors that undo each row's scale (C[r][c] * rsA[r] * rsB[c]).
int gemm_tc_store_scaled(const void *planesA, int64_t nA, const void *planesB, int64_t nB,
                         int64_t kpad, const float *rsA, const float *rsB, float *C, int64_t ldc,
                         cudaStream_t s);

// kendall.cu: batched problems.  Masks of problem i start at mask_off
// (uint2 words, K = Dr * Wn per variable); untied counts at var_off.  d_T
// holds 2 * total_vars 8-byte slots: the untied counts, then their roots.
struct KendallBatchProblem {
  const float *X;  // variable-major p x n
  int64_t p, n, Dr, Wn, K;
  int64_t mask_off, var_off;
  double *out;     // p x p, [y*p + x]
};
int kendall_batch_launch(const KendallBatchProblem *d_probs, const int64_t *d_var_prefix,
                         int64_t nprob, int64_t total_vars, const int64_t *d_tile_prefix,
                         const int64_t *d_cta_tiles, const int64_t *d_cta_off, int64_t ncta,
                         uint2 *d_masks, unsigned long long *d_T, cudaStream_t s);

// gram_tc.cu: batched cor(x) on tcgen05 (see pearson_batch_prepare).
int pearson_batch_prepare(const gt_cor_problem *probs, int64_t count, int kind, int bk,
                          int64_t chunk_elems, const std::function<int(size_t, void **)> &alloc,
                          std::function<int(cudaStream_t)> *run, int64_t *ntiles_out,
                          int64_t *nctas_out, int **err_out);

}  // namespace gt
