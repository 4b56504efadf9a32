/*
 * oracle.h -- FP64 CPU restatement of gputools' all-pairs statistics.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; it is the checker that tests/, bench.py's CPU-baseline leg
 * and __graft_entry__.smoke() compare the CUDA path against.
 *
 * Semantics restated (all arithmetic in double on float32 inputs, the way R's
 * .C call hands gputools `as.single(...)` copies):
 *   dist    : R stats::dist for the six gputools methods, as the reference's
 *             kernels compute them (inst/cuda/distance.cu:40-78 euclidean,
 *             :116-154 maximum, :192-232 manhattan, :273-316 canberra,
 *             :366-415 binary, :453-493 minkowski) with R's documented
 *             handling of 0/0 canberra terms (omitted, sum rescaled).
 *   pearson : R stats::cor(method="pearson") with use = "everything" or
 *             "pairwise.complete.obs", the quantities that src/correlation.cpp:66-161
 *             pmcc() returns (pairs, coefficients) plus the t-score rule of
 *             src/correlation.cpp:51-64 hostSignif().
 *   kendall : R stats::cor(method="kendall") = tau-b from exact integer
 *             counts, S / (sqrt(Tx) * sqrt(Ty)) clamped to [-1, 1]; the
 *             reference kernel inst/cuda/kendall.cu:4-47 computes a tau-a
 *             variant instead, and the counts exposed here let tests check
 *             both.
 *   ttest   : src/correlation.cpp:17-49 testSignif / inst/cuda/correlation.cu:294-313.
 *   mi      : B-spline mutual information, src/mi.cpp:14-164 with
 *             inst/cuda/mi.cu:1-152 (knots, min-max scaling in float, the
 *             Cox-de Boor weights, entropies and MI in log2).
 *
 * Layouts follow the reference: points row-major N x D (src/distance.h:10-26),
 * distances d[y*N + x]; correlation inputs variable-contiguous (A[x*n + k]),
 * Pearson outputs [x*nb + y] (inst/cuda/correlation.cu:149), Kendall output
 * [y*nx + x] (inst/cuda/kendall.cu:45).
 */
#ifndef GPUTOOLS_ORACLE_H
#define GPUTOOLS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_EUCLIDEAN = 0, ORC_MAXIMUM = 1, ORC_MANHATTAN = 2,
  ORC_CANBERRA = 3, ORC_BINARY = 4, ORC_MINKOWSKI = 5
};

void orc_set_threads(int nthreads);
int orc_get_threads(void);

/* out[y*na + x] = d(a_x, b_y); a and b are row-major (na x dim), (nb x dim). */
int orc_dist(const float *a, int64_t na, const float *b, int64_t nb,
             int64_t dim, int method, double p, double *out);

/* use: 0 = everything, 1 = pairwise.complete.obs.  A[x*n+k], B[y*n+k].
 * corr/pairs/ts[x*nb + y].  Any output pointer may be NULL. */
int orc_pearson(int use, const float *A, int64_t na, const float *B,
                int64_t nb, int64_t n, double *corr, double *pairs,
                double *ts);

/* tau-b; out[y*nx + x].  same != 0 means X and Y are one data set, so the
 * diagonal is exactly 1 (R's cor(x) form).  S/Tx/Ty may be NULL; when given
 * they receive S = sum sign(dx)*sign(dy) over i<j, and the untied-pair counts
 * of x and y, at [y*nx + x]. */
int orc_kendall(const float *X, int64_t nx, const float *Y, int64_t ny,
                int64_t n, int same, double *out, int64_t *S, int64_t *Tx,
                int64_t *Ty);

/* t = r * sqrt((pairs - 2) / (1 - r^2)) elementwise. */
void orc_ttest(const double *pairs, const double *r, int64_t len, double *out);

/* The hostSignif rule: r >= 0.999 -> 10000, else the t formula. */
void orc_signif(const double *pairs, const double *r, int64_t len,
                double *out);

/* Adjoints (no counterpart in the reference; see oracle.c). */
int orc_cor_backward(const float *X, int64_t p, int64_t n, const double *G,
                     double *dX);
int orc_dist_backward(const float *X, int64_t n, int64_t dim, const double *G,
                      double *dX);
int orc_mds_stress(const float *X, int64_t n, int64_t dim, const float *delta,
                   double *loss, double *dX);

/* B-spline mutual information (src/mi.cpp, inst/cuda/mi.cu): out[y*nx + x]
 * = MI(X_x, Y_y) over n samples (variables contiguous, X[x*n + k]); hx, hy
 * (may be NULL) receive the entropies.  See oracle.c for the restatement. */
int orc_bspline_mi(int nbins, int order, int64_t n, const float *X, int64_t nx,
                   const float *Y, int64_t ny, double *out, double *hx, double *hy);

/* Hierarchical clustering as the reference's kernels do it (see oracle.c):
 * D the full n x n float matrix (read only); sub/sup/val receive n - 1 steps.
 * orc_hc_method maps a method name as getClusterEnum does; lambda and beta
 * are 0.5 in every reference entry point. */
int orc_hc_method(const char *name);
float orc_hc_update(int method, float top, float bot, float nr, float np, float nk, float val,
                    float lambda, float beta);
int orc_hclust(const float *D, int64_t n, int method, float lambda, float beta, int *sub,
               int *sup, float *val);
/* formatClustering (src/rinterface.cpp): merge (len x 2, column-major) and
 * the 1-based dendrogram order of len + 1 points. */
void orc_format_clustering(int len, const int *sub, const int *sup, int *merge, int *order);

#ifdef __cplusplus
}
#endif
#endif
