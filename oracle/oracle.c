/*
 * oracle.c -- FP64 CPU restatement of gputools' all-pairs statistics.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, by bench.py's CPU-baseline leg and
 * by __graft_entry__.smoke() as the checker.  The shipped library never links
 * or calls it.  See oracle.h for the semantics and the reference lines each
 * function follows.
 *
 * Sums use Neumaier compensation so the oracle is accurate to a few ulp of
 * double, far below the float32 tolerances the CUDA path is held to.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void orc_set_threads(int nthreads) { g_threads = nthreads; }

int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* Neumaier-compensated accumulator. */
typedef struct { double s, c; } ksum;
static inline void ks_add(ksum *k, double v) {
  double t = k->s + v;
  if (!isfinite(t)) { k->s = t; return; }  /* Inf/NaN: no compensation */
  if (fabs(k->s) >= fabs(v)) k->c += (k->s - t) + v;
  else k->c += (v - t) + k->s;
  k->s = t;
}
static inline double ks_val(const ksum *k) { return k->s + k->c; }

/* ---------------------------------------------------------------- dist --- */

/* One distance between two float32 vectors of length dim, in double.
 * euclidean  sqrt(sum (a-b)^2)              distance.cu:40-78
 * maximum    max |a-b|                      distance.cu:116-154
 * manhattan  sum |a-b|                      distance.cu:192-232
 * canberra   sum |a-b|/|a+b|                distance.cu:273-316; terms with
 *            a zero numerator and zero denominator are omitted and the sum is
 *            scaled by dim/used (R ?dist); no term used -> NaN.
 * binary     #(on xor) / #(on or), 0 when no bit is on  distance.cu:366-415
 * minkowski  (sum |a-b|^p)^(1/p)            distance.cu:453-493
 */
static double dist1(const float *a, const float *b, int64_t dim, int method,
                    double p) {
  ksum acc = {0.0, 0.0};
  switch (method) {
  case ORC_EUCLIDEAN:
    for (int64_t k = 0; k < dim; k++) {
      double t = (double)a[k] - (double)b[k];
      ks_add(&acc, t * t);
    }
    return sqrt(ks_val(&acc));
  case ORC_MAXIMUM: {
    double m = 0.0;
    for (int64_t k = 0; k < dim; k++) {
      double t = fabs((double)a[k] - (double)b[k]);
      if (t > m) m = t;
    }
    return m;
  }
  case ORC_MANHATTAN:
    for (int64_t k = 0; k < dim; k++)
      ks_add(&acc, fabs((double)a[k] - (double)b[k]));
    return ks_val(&acc);
  case ORC_CANBERRA: {
    int64_t used = 0;
    for (int64_t k = 0; k < dim; k++) {
      double num = fabs((double)a[k] - (double)b[k]);
      double den = fabs((double)a[k] + (double)b[k]);
      if (num == 0.0 && den == 0.0) continue;
      ks_add(&acc, num / den);
      used++;
    }
    if (used == 0) return NAN;
    double s = ks_val(&acc);
    if (used < dim) s = s / ((double)used / (double)dim);
    return s;
  }
  case ORC_BINARY: {
    int64_t either = 0, onlyone = 0;
    for (int64_t k = 0; k < dim; k++) {
      int x = a[k] != 0.0f, y = b[k] != 0.0f;
      either += (x | y);
      onlyone += (x ^ y);
    }
    return either ? (double)onlyone / (double)either : 0.0;
  }
  case ORC_MINKOWSKI:
    for (int64_t k = 0; k < dim; k++)
      ks_add(&acc, pow(fabs((double)a[k] - (double)b[k]), p));
    return pow(ks_val(&acc), 1.0 / p);
  default:
    return NAN;
  }
}

int orc_dist(const float *a, int64_t na, const float *b, int64_t nb,
             int64_t dim, int method, double p, double *out) {
  if (method < ORC_EUCLIDEAN || method > ORC_MINKOWSKI) return -1;
  if (na < 0 || nb < 0 || dim < 0) return -2;
#pragma omp parallel for schedule(dynamic, 4) num_threads(orc_get_threads())
  for (int64_t y = 0; y < nb; y++)
    for (int64_t x = 0; x < na; x++)
      out[y * na + x] = dist1(a + x * dim, b + y * dim, dim, method, p);
  return 0;
}

/* ------------------------------------------------------------- pearson --- */

/* r, and the pair count, for one pair of variables.
 * everything  (correlation.cu:152-292 NoTest kernels): every observation is
 *             used, any NaN makes r NaN, pairs = n.
 * pairwise    (correlation.cu:7-150): observations where either value is NaN
 *             are dropped; pairs = the number kept; fewer than 2 -> NaN.
 * Two-pass: means first, then centred second moments, all in double.  A zero
 * variance gives NaN (R returns NA for it). */
static double pearson1(int use, const float *x, const float *y, int64_t n,
                       double *npairs) {
  ksum sx = {0, 0}, sy = {0, 0};
  int64_t cnt = 0;
  int has_nan = 0;
  for (int64_t k = 0; k < n; k++) {
    double a = x[k], b = y[k];
    if (isnan(a) || isnan(b)) {
      has_nan = 1;
      if (use == 1) continue;
    }
    ks_add(&sx, a);
    ks_add(&sy, b);
    cnt++;
  }
  if (use == 0) {
    *npairs = (double)n;
    if (has_nan) return NAN;
  } else {
    *npairs = (double)cnt;
  }
  if (cnt < 2) return NAN;
  double mx = ks_val(&sx) / (double)cnt, my = ks_val(&sy) / (double)cnt;
  ksum sxx = {0, 0}, syy = {0, 0}, sxy = {0, 0};
  for (int64_t k = 0; k < n; k++) {
    double a = x[k], b = y[k];
    if (isnan(a) || isnan(b)) continue;
    double da = a - mx, db = b - my;
    ks_add(&sxx, da * da);
    ks_add(&syy, db * db);
    ks_add(&sxy, da * db);
  }
  double vx = ks_val(&sxx), vy = ks_val(&syy);
  if (vx == 0.0 || vy == 0.0) return NAN;
  double r = ks_val(&sxy) / (sqrt(vx) * sqrt(vy));
  if (r > 1.0) r = 1.0;
  if (r < -1.0) r = -1.0;
  return r;
}

int orc_pearson(int use, const float *A, int64_t na, const float *B,
                int64_t nb, int64_t n, double *corr, double *pairs,
                double *ts) {
  if (use != 0 && use != 1) return -1;
  if (na < 0 || nb < 0 || n < 0) return -2;
#pragma omp parallel for collapse(2) schedule(dynamic, 64) num_threads(orc_get_threads())
  for (int64_t x = 0; x < na; x++) {
    for (int64_t y = 0; y < nb; y++) {
      double np;
      double r = pearson1(use, A + x * n, B + y * n, n, &np);
      int64_t o = x * nb + y;
      if (corr) corr[o] = r;
      if (pairs) pairs[o] = np;
      if (ts) orc_signif(&np, &r, 1, ts + o);
    }
  }
  return 0;
}

void orc_ttest(const double *pairs, const double *r, int64_t len,
               double *out) {
  for (int64_t i = 0; i < len; i++)
    out[i] = r[i] * sqrt((pairs[i] - 2.0) / (1.0 - r[i] * r[i]));
}

/* src/correlation.cpp:51-64: r at or above 0.999 reports the sentinel 10000. */
void orc_signif(const double *pairs, const double *r, int64_t len,
                double *out) {
  for (int64_t i = 0; i < len; i++) {
    if (r[i] >= 0.999) out[i] = 10000.0;
    else out[i] = r[i] * sqrt((pairs[i] - 2.0) / (1.0 - r[i] * r[i]));
  }
}

/* ------------------------------------------------------------- kendall --- */

static inline int sgn(float a, float b) { return (b > a) - (b < a); }

/* S = sum_{i<j} sign(x_j - x_i) sign(y_j - y_i); Tx, Ty = untied pairs. */
static void kendall_counts(const float *x, const float *y, int64_t n,
                           int64_t *S, int64_t *Tx, int64_t *Ty) {
  int64_t s = 0, tx = 0, ty = 0;
  for (int64_t i = 0; i < n; i++) {
    for (int64_t j = i + 1; j < n; j++) {
      int a = sgn(x[i], x[j]), b = sgn(y[i], y[j]);
      s += a * b;
      tx += a * a;
      ty += b * b;
    }
  }
  *S = s;
  *Tx = tx;
  *Ty = ty;
}

/* tau-b exactly as R evaluates it: S / (sqrt(Tx) * sqrt(Ty)), clamped. */
static double taub(int64_t S, int64_t Tx, int64_t Ty) {
  if (Tx == 0 || Ty == 0) return NAN;
  double r = (double)S / (sqrt((double)Tx) * sqrt((double)Ty));
  if (r > 1.0) r = 1.0;
  if (r < -1.0) r = -1.0;
  return r;
}

int orc_kendall(const float *X, int64_t nx, const float *Y, int64_t ny,
                int64_t n, int same, double *out, int64_t *S, int64_t *Tx,
                int64_t *Ty) {
  if (nx < 0 || ny < 0 || n < 0) return -2;
#pragma omp parallel for schedule(dynamic, 1) num_threads(orc_get_threads())
  for (int64_t y = 0; y < ny; y++) {
    for (int64_t x = 0; x < nx; x++) {
      int64_t s, tx, ty;
      kendall_counts(X + x * n, Y + y * n, n, &s, &tx, &ty);
      int64_t o = y * nx + x;
      if (S) S[o] = s;
      if (Tx) Tx[o] = tx;
      if (Ty) Ty[o] = ty;
      if (out) out[o] = (same && x == y) ? 1.0 : taub(s, tx, ty);
    }
  }
  return 0;
}

/* ------------------------------------------------------------ adjoints --- */
/* No counterpart in the reference: the adjoints of the all-pairs statistics
 * (dL/dX from an upstream dL/dC), restated from the calculus in FP64.
 *
 * Pearson, C = cor(X), variables x_j (columns, X[j*n + k]):
 *   c_j = x_j - mean(x_j), s_j = |c_j|, z_j = c_j / s_j, C_ij = z_i . z_j
 *   w_j = sum_i (G_ij + G_ji) z_i
 *   dL/dx_j = (w_j - z_j (z_j . w_j)) / s_j      (w_j and z_j have zero mean)
 * G is row-major p x p, G[i*p + j] = dL/dC_ij.  Constant variables get 0. */
int orc_cor_backward(const float *X, int64_t p, int64_t n, const double *G,
                     double *dX) {
  double *Z = (double *)malloc(sizeof(double) * (size_t)(p * n));
  double *inv = (double *)malloc(sizeof(double) * (size_t)p);
  if (!Z || !inv) { free(Z); free(inv); return -3; }
#pragma omp parallel for num_threads(orc_get_threads())
  for (int64_t j = 0; j < p; j++) {
    ksum s = {0, 0};
    for (int64_t k = 0; k < n; k++) ks_add(&s, X[j * n + k]);
    double m = ks_val(&s) / (double)n;
    ksum q = {0, 0};
    for (int64_t k = 0; k < n; k++) {
      double d = X[j * n + k] - m;
      ks_add(&q, d * d);
    }
    double nrm = sqrt(ks_val(&q));
    inv[j] = nrm > 0 ? 1.0 / nrm : 0.0;
    for (int64_t k = 0; k < n; k++) Z[j * n + k] = (X[j * n + k] - m) * inv[j];
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(orc_get_threads())
  for (int64_t j = 0; j < p; j++) {
    double *w = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < p; i++) {
      double g = G[i * p + j] + G[j * p + i];
      if (g == 0.0) continue;
      for (int64_t k = 0; k < n; k++) w[k] += g * Z[i * n + k];
    }
    ksum zw = {0, 0};
    for (int64_t k = 0; k < n; k++) ks_add(&zw, Z[j * n + k] * w[k]);
    double d = ks_val(&zw);
    for (int64_t k = 0; k < n; k++)
      dX[j * n + k] = (w[k] - Z[j * n + k] * d) * inv[j];
    free(w);
  }
  free(Z);
  free(inv);
  return 0;
}

/* Euclidean distances, D_ij = |x_i - x_j| (X row-major n x dim):
 *   dL/dx_i = sum_j (G_ij + G_ji) (x_i - x_j) / D_ij,  terms with D_ij = 0 are 0.
 * G is n x n, G[i*n + j] = dL/dD_ij. */
int orc_dist_backward(const float *X, int64_t n, int64_t dim, const double *G,
                      double *dX) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(orc_get_threads())
  for (int64_t i = 0; i < n; i++) {
    for (int64_t k = 0; k < dim; k++) dX[i * dim + k] = 0.0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double d2 = 0.0;
      for (int64_t k = 0; k < dim; k++) {
        double t = (double)X[i * dim + k] - (double)X[j * dim + k];
        d2 += t * t;
      }
      double d = sqrt(d2);
      if (d == 0.0) continue;
      double w = (G[i * n + j] + G[j * n + i]) / d;
      for (int64_t k = 0; k < dim; k++)
        dX[i * dim + k] += w * ((double)X[i * dim + k] - (double)X[j * dim + k]);
    }
  }
  return 0;
}

/* MDS stress against targets delta (R dist layout, entry (i > j) at
 * n*j - j*(j+1)/2 + i - j - 1): L = sum_{i<j} (D_ij - delta_ij)^2 and
 * dL/dx_i = sum_{j != i} 2 (D_ij - delta_ij) (x_i - x_j) / D_ij. */
int orc_mds_stress(const float *X, int64_t n, int64_t dim, const float *delta,
                   double *loss, double *dX) {
  double total = 0.0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total) num_threads(orc_get_threads())
  for (int64_t i = 0; i < n; i++) {
    if (dX)
      for (int64_t k = 0; k < dim; k++) dX[i * dim + k] = 0.0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double d2 = 0.0;
      for (int64_t k = 0; k < dim; k++) {
        double t = (double)X[i * dim + k] - (double)X[j * dim + k];
        d2 += t * t;
      }
      double d = sqrt(d2);
      int64_t a = i > j ? i : j, b = i > j ? j : i;
      double del = delta[n * b - b * (b + 1) / 2 + a - b - 1];
      if (j > i) total += (d - del) * (d - del);
      if (dX && d > 0.0) {
        double w = 2.0 * (d - del) / d;
        for (int64_t k = 0; k < dim; k++)
          dX[i * dim + k] += w * ((double)X[i * dim + k] - (double)X[j * dim + k]);
      }
    }
  }
  if (loss) *loss = total;
  return 0;
}

/* ------------------------------------------------------ mutual information --- */
/* B-spline mutual information (R/gpuMi.R, src/mi.cpp, inst/cuda/mi.cu).
 *
 * Knots (src/mi.cpp:14-30 initKnots): order zeros, then 1, 2, ... up to
 * index nbins - 1, then the last value + 1 repeated; nknots = nbins + order.
 * Each variable is scaled to [0, knot_max] from its own min and max, in float
 * as inst/cuda/mi.cu:3-25 scale() does (a variable whose max equals its min
 * has no scale there -- 0/0 -- and is taken as all zeros here).  Its samples'
 * B-spline weights follow the Cox-de Boor recursion with the index bounds of
 * inst/cuda/mi.cu:39-86 get_bin_scores, here in double.  Entropies
 * (inst/cuda/mi.cu:88-113) and mutual information (inst/cuda/mi.cu:115-152)
 * use probabilities p = (sum of weights) / nsamples and log2, with p <= 0
 * contributing nothing:
 *   H(x)    = -sum_a p_a log2 p_a
 *   MI(x,y) = sum_ab p_ab log2 p_ab + H(x) + H(y),  p_ab = sum_k wx_ka wy_kb / n. */
static double mi_frac(double numer, double denom) {
  if (numer == denom && numer != 0.0) return 1.0;
  if (denom != 0.0) return numer / denom;
  return 0.0;
}

/* weights w[k * nbins + a] of variable x (n samples) */
static void mi_weights(const float *x, int64_t n, int nbins, int order, const float *knots,
                       int nknots, double *w) {
  float mn = x[0], mx = x[0];
  for (int64_t k = 1; k < n; k++) {
    if (x[k] < mn) mn = x[k];
    if (x[k] > mx) mx = x[k];
  }
  const float kmax = knots[nknots - 1];
  const float delta = mx - mn;
  memset(w, 0, sizeof(double) * (size_t)n * (size_t)nbins);
  for (int64_t k = 0; k < n; k++) {
    const float z = delta > 0.f ? (kmax * (x[k] - mn)) / delta : 0.f;
    double *b = w + k * nbins;
    int i0 = (int)floorf(z) + order - 1;
    if (i0 >= nbins) i0 = nbins - 1;
    b[i0] = 1.0;
    for (int i = 2; i <= order; i++) {
      for (int j = i0 - i + 1; j <= i0; j++) {
        double t1, t2;
        if (j < 0 || j >= nbins || j >= nknots || j + i - 1 < 0 || j > nknots)
          t1 = 0.0;
        else
          t1 = mi_frac((double)z - knots[j], (double)knots[j + i - 1] - knots[j]) * b[j];
        if (j + 1 < 0 || j + 1 >= nbins || j + 1 >= nknots || j + i < 0 || j + i >= nknots)
          t2 = 0.0;
        else
          t2 = mi_frac((double)knots[j + i] - z, (double)knots[j + i] - knots[j + 1]) * b[j + 1];
        b[j] = t1 + t2;
      }
    }
  }
}

static double plog2p(double p) { return p > 0.0 ? p * log2(p) : 0.0; }

int orc_bspline_mi(int nbins, int order, int64_t n, const float *X, int64_t nx,
                   const float *Y, int64_t ny, double *out, double *hx, double *hy) {
  if (nbins < 1 || order < 1 || order > nbins || n < 1 || nx < 0 || ny < 0) return -1;
  const int nknots = nbins + order;
  float *knots = (float *)malloc(sizeof(float) * (size_t)nknots);
  const int degree = nbins - 1;
  for (int i = 0; i < nknots; i++) {
    if (i <= order - 1) knots[i] = 0.f;
    else if (i <= degree) knots[i] = knots[i - 1] + 1.f;
    else knots[i] = knots[degree] + 1.f;
  }
  double *wx = (double *)malloc(sizeof(double) * (size_t)(nx * n * nbins));
  double *wy = (double *)malloc(sizeof(double) * (size_t)(ny * n * nbins));
  double *ex = (double *)malloc(sizeof(double) * (size_t)(nx > 0 ? nx : 1));
  double *ey = (double *)malloc(sizeof(double) * (size_t)(ny > 0 ? ny : 1));
  if (!knots || !wx || !wy || !ex || !ey) {
    free(knots); free(wx); free(wy); free(ex); free(ey);
    return -3;
  }
  const float *src[2] = {X, Y};
  double *w[2] = {wx, wy}, *e[2] = {ex, ey};
  const int64_t cnt[2] = {nx, ny};
  for (int s = 0; s < 2; s++) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(orc_get_threads())
    for (int64_t v = 0; v < cnt[s]; v++) {
      double *wv = w[s] + v * n * nbins;
      mi_weights(src[s] + v * n, n, nbins, order, knots, nknots, wv);
      double h = 0.0;
      for (int a = 0; a < nbins; a++) {
        ksum acc = {0.0, 0.0};
        for (int64_t k = 0; k < n; k++) ks_add(&acc, wv[k * nbins + a]);
        h -= plog2p(ks_val(&acc) / (double)n);
      }
      e[s][v] = h;
    }
  }
#pragma omp parallel for collapse(2) schedule(dynamic, 16) num_threads(orc_get_threads())
  for (int64_t y = 0; y < ny; y++) {
    for (int64_t x = 0; x < nx; x++) {
      const double *a = wx + x * n * nbins, *b = wy + y * n * nbins;
      double mi = 0.0;
      for (int i = 0; i < nbins; i++) {
        for (int j = 0; j < nbins; j++) {
          ksum acc = {0.0, 0.0};
          for (int64_t k = 0; k < n; k++) ks_add(&acc, a[k * nbins + i] * b[k * nbins + j]);
          mi += plog2p(ks_val(&acc) / (double)n);
        }
      }
      out[y * nx + x] = mi + ex[x] + ey[y];
    }
  }
  if (hx) memcpy(hx, ex, sizeof(double) * (size_t)nx);
  if (hy) memcpy(hy, ey, sizeof(double) * (size_t)ny);
  free(knots); free(wx); free(wy); free(ex); free(ey);
  return 0;
}

/* ------------------------------------------------- hierarchical clustering --- */
/* gpuHclust / gpuDistClust (R/gpuHclust.R:41-146): the reference's loop of
 * src/hcluster.cpp:40-201 over the kernels of inst/cuda/hcluster.cu, on the
 * full n x n float matrix, with the diagonal set to +inf:
 *   per active row (count > 0) the minimum over columns 0..row, ties broken
 *   as its 32-thread strided scan and tree reduction break them (smallest
 *   column mod 32, then smallest column: find_min1_kernel, :11-59); the
 *   winning row likewise over the rows' minima (find_min2_kernel, :61-106);
 *   sub = the winning column, sup = the winning row, val = the minimum,
 *   count[sup] += count[sub], count[sub] = -count[sub]; then the row and
 *   column of sup get the linkage update and those of sub +inf (:108-401).
 * The update expressions are evaluated as written there (float, with the
 * double promotions of the 2.0 / 4.0 / 1.0 - lambda constants), each
 * operation rounded on its own (no fused multiply-add; the reference's
 * run-time compilation leaves that choice to its compiler).  Methods follow
 * getClusterEnum (src/rinterface.cpp): an unknown name -- among them R's
 * "flexible group", which the reference matches against "flexible_group" --
 * is single linkage. */
enum { HC_SINGLE = 0, HC_COMPLETE, HC_WPGMA, HC_AVERAGE, HC_MEDIAN, HC_CENTROID,
       HC_FLEXIBLE_GROUP, HC_FLEXIBLE, HC_WARD, HC_MCQUITTY };

int orc_hc_method(const char *name) {
  static const char *names[] = {"complete", "wpgma", "average", "median", "centroid",
                                "flexible_group", "flexible", "ward", "mcquitty"};
  static const int ids[] = {HC_COMPLETE, HC_WPGMA, HC_AVERAGE, HC_MEDIAN, HC_CENTROID,
                            HC_FLEXIBLE_GROUP, HC_FLEXIBLE, HC_WARD, HC_MCQUITTY};
  for (int i = 0; i < 9; i++)
    if (name && strcmp(name, names[i]) == 0) return ids[i];
  return HC_SINGLE;
}

/* (v1, c1) before (v2, c2): the value, then column mod 32, then column; a
 * NaN is never before anything. */
static int hc_before(float v1, int64_t c1, float v2, int64_t c2) {
  if (v1 < v2) return 1;
  if (!(v1 == v2)) return 0;
  if ((c1 & 31) != (c2 & 31)) return (c1 & 31) < (c2 & 31);
  return c1 < c2;
}

float orc_hc_update(int method, float top, float bot, float nr, float np, float nk, float val,
                    float lambda, float beta) {
  const float nq = nr - np;
  switch (method) {
    case HC_COMPLETE: return top > bot ? top : (bot == bot ? bot : top);
    case HC_WPGMA:
    case HC_MCQUITTY: return (float)((double)(bot + top) / 2.0);
    case HC_AVERAGE: {
      const float a = top * np, b = bot * nq;
      return (a + b) / nr;
    }
    case HC_MEDIAN: return (float)((double)(bot + top) / 2.0 - (double)val / 4.0);
    case HC_CENTROID: {
      const float a = top * np, b = bot * nq;
      const float t1 = (a + b) / nr;
      const float pq = np * nq, num = pq * val, den = nr * nr;
      return t1 - num / den;
    }
    case HC_FLEXIBLE_GROUP: {
      const double l1 = 1.0 - (double)lambda;
      const double a = ((double)bot * l1) * (double)np, b = ((double)top * l1) * (double)nq;
      const float bv = beta * val;
      return (float)((a + b) / (double)nr + (double)bv);
    }
    case HC_FLEXIBLE: {
      const double l1 = 1.0 - (double)lambda;
      const double a = (double)bot * l1, b = (double)top * l1;
      const float bv = beta * val;
      return (float)((a + b) / 2.0 + (double)bv);
    }
    case HC_WARD: {
      const float a = bot * (np + nk), b = top * (nq + nk), c = val * nk;
      float r = ((a + b) - c) / (nr + nk);
      if (isinf(r)) r = INFINITY;
      return r;
    }
    default: return bot < top ? bot : (top == top ? top : bot);  /* single: fminf */
  }
}

int orc_hclust(const float *D, int64_t n, int method, float lambda, float beta, int *sub,
               int *sup, float *val) {
  if (n < 2) return -1;
  float *d = (float *)malloc(sizeof(float) * (size_t)(n * n));
  float *cnt = (float *)malloc(sizeof(float) * (size_t)n);
  float *mv = (float *)malloc(sizeof(float) * (size_t)n);
  int64_t *mc = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  if (!d || !cnt || !mv || !mc) {
    free(d); free(cnt); free(mv); free(mc);
    return -3;
  }
  memcpy(d, D, sizeof(float) * (size_t)(n * n));
  for (int64_t i = 0; i < n; i++) {
    d[i * n + i] = INFINITY;
    cnt[i] = 1.f;
  }
  for (int64_t it = 0; it + 1 < n; it++) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(orc_get_threads())
    for (int64_t row = 0; row < n; row++) {
      float bv = INFINITY;
      int64_t bc = 0;
      if (cnt[row] > 0.f) {
        for (int64_t col = 0; col <= row; col++) {
          const float t = d[row * n + col];
          if (hc_before(t, col, bv, bc)) { bv = t; bc = col; }
        }
      }
      mv[row] = bv;
      mc[row] = bc;
    }
    float bv = INFINITY;
    int64_t br = 0;
    for (int64_t row = 0; row < n; row++)
      if (cnt[row] > 0.f && hc_before(mv[row], row, bv, br)) { bv = mv[row]; br = row; }
    const int64_t c = mc[br], r = br;
    sub[it] = (int)c;
    sup[it] = (int)r;
    val[it] = bv;
    cnt[r] += cnt[c];
    cnt[c] = -cnt[c];
    const float nr = cnt[r], np = -cnt[c];
    for (int64_t col = 0; col < n; col++) {
      const float top = d[c * n + col], bot = d[r * n + col];
      float nv = orc_hc_update(method, top, bot, nr, np, cnt[col], bv, lambda, beta);
      if (col == c || col == r || (method == HC_WARD && nr == -cnt[col])) nv = INFINITY;
      d[r * n + col] = nv;
      d[col * n + r] = nv;
    }
    for (int64_t col = 0; col < n; col++) {
      d[c * n + col] = INFINITY;
      d[col * n + c] = INFINITY;
    }
  }
  free(d); free(cnt); free(mv); free(mc);
  return 0;
}

/* formatClustering + getPrintOrder (src/rinterface.cpp): R's merge matrix
 * (column-major len x 2; -(i+1) a point, j+1 the cluster of step j) and the
 * dendrogram order, the depth-first walk kept on an explicit stack. */
void orc_format_clustering(int len, const int *sub, const int *sup, int *merge, int *order) {
  for (int i = 0; i < len; i++) {
    merge[i] = -(sub[i] + 1);
    merge[i + len] = -(sup[i] + 1);
  }
  for (int i = 0; i < len; i++) {
    for (int j = i + 1; j < len; j++) {
      if (merge[j] == merge[i] || merge[j] == merge[i + len]) merge[j] = i + 1;
      if (merge[j + len] == merge[i] || merge[j + len] == merge[i + len]) merge[j + len] = i + 1;
      if ((merge[j + len] < 0 && merge[j] > 0) ||
          (merge[j] > 0 && merge[j + len] > 0 && merge[j] > merge[j + len])) {
        const int h = merge[j];
        merge[j] = merge[j + len];
        merge[j + len] = h;
      }
    }
  }
  if (len < 1) return;
  int *stack = (int *)malloc(sizeof(int) * (size_t)(2 * len + 2));
  int top = 0, otop = len;
  stack[top++] = len - 1;
  while (top > 0) {
    const int level = stack[--top];
    /* the recursion visits the right child, then the left: push left first */
    const int left = merge[level], right = merge[level + len];
    if (left < 0) stack[top++] = -1 - (-left);  /* leaf marker: -(point + 2) */
    else stack[top++] = left - 1;
    if (right < 0) stack[top++] = -1 - (-right);
    else stack[top++] = right - 1;
    while (top > 0 && stack[top - 1] < 0) {
      order[otop--] = -(stack[--top] + 1);
    }
  }
  free(stack);
}
