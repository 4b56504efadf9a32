/*
 * gputools_gb300.h -- C ABI of libgputools_gb300.so, the GB300 (sm_103a)
 * implementation of gputools' all-pairs hot path (gpuDist, gpuCor, gpuTtest)
 * and the statistics built on it (gpuMi, gpuHclust / gpuDistClust).
 *
 * Two layers:
 *
 *  1. The reference's own `.C` entry points, same names, argument order and
 *     meaning, so R's `useDynLib` + `.C("Rdistances", ...)` etc. bind to this
 *     library unchanged.  They are synchronous, take host buffers, and report
 *     errors through R's error() when the library is loaded into R (resolved
 *     weakly at run time, after every device buffer is released), otherwise
 *     through gt_last_error().
 *
 *  2. gt_* functions that return a status code (GT_OK = 0) for non-R callers,
 *     with host-buffer and device-buffer variants.  Device variants take raw
 *     device pointers and a cudaStream_t (passed as void*, NULL = the legacy
 *     default stream); they are asynchronous with respect to the host.
 *
 * Layouts (identical to the reference):
 *   points        row-major N x D float32, one point per row
 *                 (src/distance.h:10-26, R/gpuHclust.R:21-27 passes t(points)).
 *   distances     N x N float32, d(x, y) at [y*N + x], symmetric, zero
 *                 diagonal (src/distance.h:15-17); or, GT_LAYOUT_DIST, R's
 *                 `dist` vector: the strict lower triangle by columns,
 *                 entry (i > j) at n*j - j*(j+1)/2 + i - j - 1.
 *   correlation   inputs variable-contiguous: variable x occupies
 *                 A[x*n .. x*n + n-1] (R's column-major n x p matrix);
 *                 Pearson outputs at [x*nB + y] (inst/cuda/correlation.cu:149);
 *                 Kendall output at [y*nx + x] (inst/cuda/kendall.cu:45).
 */
#ifndef GPUTOOLS_GB300_H
#define GPUTOOLS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GT_OK 0
#define GT_EINVAL 1      /* bad argument (size, method name, pointer)        */
#define GT_ECUDA 2       /* a CUDA runtime call failed                       */
#define GT_ENOMEM 3      /* device workspace could not be allocated          */
#define GT_ENODEV 4      /* no usable CUDA device                            */
#define GT_ETIMEOUT 5    /* a bounded device-side wait gave up               */
#define GT_EUNSUPPORTED 6 /* valid request this build does not support       */

/* ---- enums -------------------------------------------------------------- */
/* src/distance.h:5-8 dist_method, same order. */
enum gt_dist_method {
  GT_EUCLIDEAN = 0, GT_MAXIMUM = 1, GT_MANHATTAN = 2,
  GT_CANBERRA = 3, GT_BINARY = 4, GT_MINKOWSKI = 5
};
/* src/correlation.h:1 UseObs, same values as rpmcc's whichObs. */
enum gt_use_obs { GT_EVERYTHING = 0, GT_PAIRWISE_COMPLETE = 1 };
enum gt_layout { GT_LAYOUT_FULL = 0, GT_LAYOUT_DIST = 1 };
/* How Pearson and Euclidean Gram contractions are evaluated. */
enum gt_gram_path {
  GT_GRAM_TC_BF16X3 = 0, /* tcgen05, each operand split hi+lo bf16, 3 products */
  GT_GRAM_TC_BF16X6 = 1, /* tcgen05, 3-way bf16 split, 6 products             */
  GT_GRAM_FP32 = 2,      /* plain FP32 CUDA-core path                         */
  GT_GRAM_TC_F16X3 = 3,  /* tcgen05, power-of-two scaled hi+lo fp16, 3 products */
  GT_GRAM_TC_F16X6 = 4   /* tcgen05, three fixed-point fp16 digits per value whose
                            products sum exactly in FP32 (error-free split),
                            6 products; Pearson only (gpuDist runs f16x3) */
};

/* ======================================================================== *
 * 1. The reference's .C entry points                                        *
 * ======================================================================== */

/* Replaces src/rinterface.cpp:206-214 (declared src/rinterface.h:53-55).
 * d(x,y) for every pair of rows of `points` (numPoints x dim, row-major) into
 * `distances` (numPoints^2, [y*N + x]).  method: "euclidean", "maximum",
 * "manhattan", "canberra", "binary", "minkowski"; any other string means
 * euclidean, as src/rinterface.cpp:147-156 getDistEnum does.  p is the
 * Minkowski power. */
void Rdistances(const float *points, const int *numPoints, const int *dim,
                float *distances, const char **method, const float *p);

/* Replaces src/rinterface.cpp:33-55 (declared src/rinterface.h:4-8).
 * whichObs 0 = "everything", 1 = "pairwise.complete.obs"; any other value is
 * an error ("unknown use method").  For every pair (x in A, y in B):
 * numPairs, correlations (Pearson r) and signifs (t-score, 10000 when
 * r >= 0.999, src/correlation.cpp:51-64) at [x*numSamplesB + y]. */
void rpmcc(const int *whichObs, const float *samplesA, const int *numSamplesA,
           const float *samplesB, const int *numSamplesB,
           const int *sampleSize, float *numPairs, float *correlations,
           float *signifs);

/* Replaces src/rinterface.cpp:128-132 (declared src/rinterface.h:41-42).
 * Kendall's tau-b (R's cor(method = "kendall")) for every pair (x in X,
 * y in Y) at answers[y*nx + x], from exact integer pair counts. */
void RgpuKendall(const float *X, const int *nx, const float *Y, const int *ny,
                 const int *sampleSize, double *answers);

/* Replaces src/rinterface.cpp:415-422 (declared src/rinterface.h:73-76;
 * R/gpuMi.R).  B-spline mutual information of every pair (x in A, y in B),
 * nsamples values per variable (variables contiguous), at
 * mutualInfo[y*rowsA + x]: nBins bins, B-splines of order splineOrder
 * (1 <= splineOrder <= min(nBins, 8)).  A variable whose values are all equal
 * is scaled to zeros (the reference divides 0 by 0 there). */
void rBSplineMutualInfo(const int *nBins, const int *splineOrder, const int *nsamples,
                        const int *rowsA, const float *A, const int *rowsB,
                        const float *B, float *mutualInfo);

/* Replaces src/rinterface.cpp:216-239 (declared src/rinterface.h:56-57;
 * R/gpuHclust.R gpuHclust).  Agglomerative clustering of the numPoints x
 * numPoints matrix distMat (R's as.matrix(dist); entry (i, j) at
 * [i*numPoints + j], only the lower triangle and the rows of merged pairs
 * are read).  merge: (numPoints-1) x 2 column-major, R's hclust convention
 * (negative = point, positive = step); order: numPoints leaves, 1-based;
 * val: merge heights.  method: "single", "complete", "average", "mcquitty",
 * "wpgma", "median", "centroid", "flexible_group", "flexible", "ward"; any
 * other string (R's "flexible group" included) means single linkage, as
 * src/rinterface.cpp:158-170 getClusterEnum does.  Lance-Williams constants
 * lambda = beta = 0.5. */
void Rhcluster(const float *distMat, const int *numPoints, int *merge, int *order,
               float *val, const char **method);

/* Replaces src/rinterface.cpp:172-204 (declared src/rinterface.h:50-52;
 * R/gpuHclust.R gpuDistClust).  Rdistances(points, distmethod, p = 2)
 * followed by Rhcluster(clustmethod); the distances never leave the device. */
void Rdistclust(const char **distmethod, const char **clustmethod, const float *points,
                const int *numPoints, const int *dim, int *merge, int *order, float *val);

/* Replace src/rinterface.cpp:79-85 (declared src/rinterface.h:23-24). */
void rsetDevice(const int *device);
void rgetDevice(int *device);

/* Replaces src/rinterface.cpp:87-91 (R/gpuCor.R:64-74 gpuTtest):
 * ts[i] = coeffs[i] * sqrt((pairs[i] - 2) / (1 - coeffs[i]^2)). */
void rtestT(const float *pairs, const float *coeffs, const int *n, float *ts);

/* Replace src/cudaUtils.cpp:118-165 and :167-195.  The reference compiles its
 * kernels with NVRTC when R loads the package (R/zzz.R:1-39); this library's
 * kernels are compiled ahead of time for sm_103a, so cuCompile only checks
 * that a device is present and unloadPackage frees the cached workspace. */
void cuCompile(const int *numFiles, const char **cuFilenames,
               const char **cuSrc);
void unloadPackage(void);

/* ======================================================================== *
 * 2. Status-returning API                                                   *
 * ======================================================================== */

/* Message of the calling thread's last failure ("" if none). */
const char *gt_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int gt_version(void);
/* Frees the device workspace of every device this thread touched. */
void gt_release_workspace(void);

/* Bounded device-side waits.  The tensor-core kernels never wait without a
 * limit: a wait that gives up makes its CTA stop, drain its copies and
 * multiplies, free its tensor memory and set the device's error word, and
 * the call's results are then incomplete.  The host-buffer entries (gt_pmcc,
 * gt_distances, gt_mutual_info, the .C entries) read the word before they
 * return and report GT_ETIMEOUT.  Device-buffer entries and batch-plan
 * launches are asynchronous and report it only through gt_device_status:
 * it synchronises `stream`, returns GT_ETIMEOUT if any such kernel on the
 * current device timed out since the last check on that device (and clears
 * the word), else GT_OK. */
int gt_device_status(void *stream);
/* Limit of each bounded wait in nanoseconds for launches made afterwards by
 * this process (0 restores the default of 2 s).  A diagnostic: a very short
 * limit makes waits give up while their work is still in flight. */
int gt_set_wait_limit_ns(uint64_t ns);
/* Number of CUDA kernels this library has launched in this process (a
 * monotone counter, for measuring how many launches a call makes). */
uint64_t gt_kernel_launches(void);

/* Kernel timing with CUDA events recorded on the launching stream around the
 * library's main kernels ("pearson_gram", "euclid_gram", "dist", "kendall_count",
 * ...).  Enabling adds two event records per timed launch.
 * gt_profile_kernel_ms waits for the recorded events and returns the summed
 * duration and the number of launches of `name` since the last reset. */
void gt_profile_enable(int on);
void gt_profile_reset(void);
int gt_profile_kernel_ms(const char *name, double *total_ms, uint64_t *launches);

/* Select the evaluation of Pearson / Euclidean Gram contractions
 * (enum gt_gram_path) for calls made afterwards by this process. */
int gt_set_gram_path(int path);
int gt_get_gram_path(void);

/* Host buffers, synchronous.  Same result as Rdistances. */
int gt_distances(const float *points, int64_t n, int64_t dim, float *out,
                 int method, float p);

/* Device buffers, asynchronous on `stream`.  layout = enum gt_layout;
 * GT_LAYOUT_FULL writes n*n floats, GT_LAYOUT_DIST n*(n-1)/2. */
int gt_distances_device(const float *d_points, int64_t n, int64_t dim,
                        float *d_out, int layout, int method, float p,
                        void *stream);

/* Host buffers, synchronous.  Same result as rpmcc; any output may be NULL. */
int gt_pmcc(int use, const float *A, int64_t nA, const float *B, int64_t nB,
            int64_t n, float *pairs, float *corr, float *ts);

/* Device buffers.  d_B == d_A (same pointer) marks the symmetric problem
 * cor(x), computed once per unordered pair and mirrored. */
int gt_pmcc_device(int use, const float *d_A, int64_t nA, const float *d_B,
                   int64_t nB, int64_t n, float *d_pairs, float *d_corr,
                   float *d_ts, void *stream);

/* No counterpart in the reference.  Same arguments and results as
 * gt_pmcc_device evaluated on CUDA cores (GT_GRAM_FP32), but it allocates no
 * device memory: for callers whose device memory belongs to another
 * allocator or a fixed budget, or who cannot afford the synchronisation an
 * allocation may bring.  Its scratch is a 64 MiB array in the library's
 * device image, which every GPU that loads the library holds until exit;
 * problems needing more scratch -- 4*(nA + nB)*round4(n) + 24*(nA + nB)
 * bytes, nB terms omitted when d_B == d_A -- are rejected with GT_EINVAL.
 * The first call on a device looks up the array's address (once per device,
 * with that device current); make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller. */
int gt_pmcc_device_noalloc(int use, const float *d_A, int64_t nA,
                           const float *d_B, int64_t nB, int64_t n,
                           float *d_pairs, float *d_corr, float *d_ts,
                           void *stream);

/* Host buffers, synchronous.  Same result as RgpuKendall. */
int gt_kendall(const float *X, int64_t nx, const float *Y, int64_t ny,
               int64_t n, double *out);

/* Device buffers; d_Y == d_X marks cor(x) (diagonal exactly 1). */
int gt_kendall_device(const float *d_X, int64_t nx, const float *d_Y,
                      int64_t ny, int64_t n, double *d_out, void *stream);

/* Host buffers, synchronous.  Same result as rBSplineMutualInfo:
 * out[y*nx + x] = MI(X_x, Y_y); Y == X (and ny == nx) is the symmetric case. */
int gt_mutual_info(int nbins, int order, int64_t n, const float *X, int64_t nx,
                   const float *Y, int64_t ny, float *out);

/* Device buffers; d_Y == d_X with ny == nx computes each unordered pair once
 * and writes both entries.  Up to 32 bins on the tensor cores (f16x3 Gram of
 * the B-spline weights), more on the CUDA cores. */
int gt_mutual_info_device(int nbins, int order, int64_t n, const float *d_X,
                          int64_t nx, const float *d_Y, int64_t ny, float *d_out,
                          void *stream);

/* Host buffers, synchronous.  Same result as Rhcluster; method as there. */
int gt_hclust(const float *dist, int64_t n, const char *method, int *merge, int *order,
              float *height);

/* Device matrix (n x n, overwritten: the merges are made in place), host
 * results; returns after the merges are done (synchronises `stream`). */
int gt_hclust_device(float *d_dist, int64_t n, const char *method, int *merge, int *order,
                     float *height, void *stream);

/* Host buffers, synchronous.  Same result as Rdistclust; dist_method is enum
 * gt_dist_method. */
int gt_distclust(const float *points, int64_t n, int64_t dim, int dist_method,
                 const char *method, int *merge, int *order, float *height);

/* src/rinterface.cpp:241-290 formatClustering on the host: the step list
 * (sub[i], sup[i]: the two 0-based row indices merged at step i, len steps)
 * to R's merge matrix and leaf order. */
int gt_hclust_format(int len, const int *sub, const int *sup, int *merge, int *order);

/* ---- adjoints (no counterpart in the reference) ------------------------- */

/* dL/dX of C = cor(X) (Pearson, "everything") given G = dL/dC.
 * X variable-major p x n (X[j*n + k]), G row-major p x p (G[i*p + j] =
 * dL/dC_ij; G and its transpose give the same result), dX like X.  Means and
 * norms are recomputed in FP64; the contraction W = (G + G^T) Z runs on the
 * selected Gram path.  Constant variables get a zero gradient. */
int gt_cor_backward_device(const float *d_X, int64_t p, int64_t n,
                           const float *d_G, float *d_dX, void *stream);

/* dL/dX of the Euclidean distances D of the rows of X (n x dim row-major)
 * given G = dL/dD (n x n, G[i*n + j]); terms with D_ij = 0 contribute 0.
 * Up to 32 dimensions, and up to 64 outside 8192..32768 points, one fused
 * CUDA-core pass (D recomputed, nothing n x n stored); otherwise D from the
 * tensor-core distance path, W = (G + G^T) / D as split-bf16 planes and W X on
 * the tensor cores (about 10 n^2 bytes of device workspace). */
int gt_dist_backward_device(const float *d_X, int64_t n, int64_t dim,
                            const float *d_G, float *d_dX, void *stream);

/* MDS stress L = sum_{i<j} (D_ij - delta_ij)^2 and dL/dX, delta in R's dist
 * layout; *d_loss (double, may be NULL) receives L.  Evaluated like
 * gt_dist_backward_device with W = 2 (D - delta) / D. */
int gt_mds_stress_device(const float *d_X, int64_t n, int64_t dim,
                         const float *d_delta, float *d_dX, double *d_loss,
                         void *stream);

/* .C-style host-buffer forms for an R gradient wrapper:
 * gpuCorBackward(x, grad), gpuDistBackward(points, grad),
 * gpuMdsStress(points, delta).  X as R's as.single(x) (n x p column-major =
 * variable-major), G as as.single(grad) (either orientation). */
void RgpuCorBackward(const float *X, const int *nobs, const int *nvar,
                     const float *G, float *dX);
void RgpuDistBackward(const float *points, const int *numPoints,
                      const int *dim, const float *G, float *dX);
void RgpuMdsStress(const float *points, const int *numPoints, const int *dim,
                   const float *delta, double *loss, float *dX);

/* ---- batches (no counterpart in the reference) --------------------------- */

/* One Pearson problem of a batch: cor(x) of a variable-major p x n device
 * matrix, outputs p x p on the device (any may be NULL), rows `ld` floats
 * apart (ld >= p; 0 means p).  A row stride that is a multiple of 8 floats
 * keeps every row on 32-byte sectors: with ld = p and p not a multiple of 8
 * the rows straddle sectors, and the partially written sectors cost the
 * output stores up to half their rate. */
typedef struct gt_cor_problem {
  const float *X;
  int64_t p, n;
  float *corr, *ts, *pairs;
  int64_t ld;
} gt_cor_problem;

/* One Kendall problem of a batch: tau-b of cor(x), out p x p doubles. */
typedef struct gt_kendall_problem {
  const float *X;
  int64_t p, n;
  double *out;
} gt_kendall_problem;

typedef struct gt_batch_plan gt_batch_plan;

/* Plan flags. */
#define GT_BATCH_NO_GRAPH 1  /* launch the kernels directly, no CUDA graph   */
#define GT_BATCH_AUTOTUNE 2  /* time the candidate tile configurations once  */

/* Build a plan for `count` problems on the current device: buffers,
 * descriptors, a host-balanced tile schedule, and (unless
 * GT_BATCH_NO_GRAPH) a CUDA graph of the launches.  Creating the plan runs
 * the batch once.  The problems' pointers must stay valid while the plan is
 * used; gt_batch_plan_launch recomputes every output from the current
 * inputs. */
int gt_pmcc_batch_plan_create(const gt_cor_problem *problems, int64_t count,
                              int flags, gt_batch_plan **plan);
int gt_kendall_batch_plan_create(const gt_kendall_problem *problems,
                                 int64_t count, int flags, gt_batch_plan **plan);
int gt_batch_plan_launch(gt_batch_plan *plan, void *stream);
const char *gt_batch_plan_describe(const gt_batch_plan *plan);
void gt_batch_plan_destroy(gt_batch_plan *plan);

/* Device buffers: t-scores as rtestT. */
int gt_ttest_device(const float *d_pairs, const float *d_coeffs, int64_t n,
                    float *d_ts, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUTOOLS_GB300_H */
