// rinterface.cu -- the reference's `.C` entry points (src/rinterface.cpp,
// declared in src/rinterface.h) on top of the status-returning gt_* API.
//
// R calls these through `.C(...)`, which passes copies of every argument and
// copies the outputs back (R/gpuHclust.R:21-27, R/gpuCor.R:34-55).  They are
// synchronous and return nothing, as in the reference.  A failure is reported
// through R's error() when the library runs inside R -- looked up as a weak
// symbol so the same shared object also loads outside R -- and only after
// every device resource of the call has been released; outside R the message
// is kept for gt_last_error() and printed to stderr.
#include "common.cuh"
#include "kernels.cuh"

#include <atomic>
#include <cstring>

extern "C" void Rf_error(const char *fmt, ...) __attribute__((weak));

namespace gt {
namespace {

std::atomic<int> g_gram_path{GT_GRAM_TC_F16X3};

// src/rinterface.cpp:147-156 getDistEnum: exact names, anything else is
// euclidean.
int dist_enum(const char *m) {
  if (!m) return GT_EUCLIDEAN;
  if (!std::strcmp(m, "maximum")) return GT_MAXIMUM;
  if (!std::strcmp(m, "manhattan")) return GT_MANHATTAN;
  if (!std::strcmp(m, "canberra")) return GT_CANBERRA;
  if (!std::strcmp(m, "binary")) return GT_BINARY;
  if (!std::strcmp(m, "minkowski")) return GT_MINKOWSKI;
  return GT_EUCLIDEAN;
}

void report(int status, const char *where) {
  if (status == GT_OK) return;
  const char *msg = last_error();
  if (Rf_error) Rf_error("%s: %s", where, msg);
  std::fprintf(stderr, "gputools_gb300: %s: %s\n", where, msg);
}

}  // namespace
}  // namespace gt

extern "C" {

int gt_set_gram_path(int path) {
  gt::clear_error();
  if (path != GT_GRAM_TC_BF16X3 && path != GT_GRAM_TC_BF16X6 && path != GT_GRAM_FP32 &&
      path != GT_GRAM_TC_F16X3 && path != GT_GRAM_TC_F16X6)
    return gt::fail(GT_EINVAL, "unknown gram path %d", path);
  gt::g_gram_path.store(path);
  return GT_OK;
}

int gt_get_gram_path(void) { return gt::g_gram_path.load(); }

void Rdistances(const float *points, const int *numPoints, const int *dim, float *distances,
                const char **method, const float *p) {
  gt::clear_error();
  int st;
  if (!numPoints || !dim || !method || !p) st = gt::fail(GT_EINVAL, "null argument");
  else st = gt_distances(points, *numPoints, *dim, distances, gt::dist_enum(*method), *p);
  gt::report(st, "Rdistances");
}

void rpmcc(const int *whichObs, const float *samplesA, const int *numSamplesA,
           const float *samplesB, const int *numSamplesB, const int *sampleSize,
           float *numPairs, float *correlations, float *signifs) {
  gt::clear_error();
  int st;
  if (!whichObs || !numSamplesA || !numSamplesB || !sampleSize) {
    st = gt::fail(GT_EINVAL, "null argument");
  } else if (*whichObs != GT_EVERYTHING && *whichObs != GT_PAIRWISE_COMPLETE) {
    // src/rinterface.cpp:47-48
    st = gt::fail(GT_EINVAL, "unknown use method");
  } else {
    st = gt_pmcc(*whichObs, samplesA, *numSamplesA, samplesB, *numSamplesB, *sampleSize,
                 numPairs, correlations, signifs);
  }
  gt::report(st, "rpmcc");
}

void RgpuKendall(const float *X, const int *nx, const float *Y, const int *ny,
                 const int *sampleSize, double *answers) {
  gt::clear_error();
  int st;
  if (!nx || !ny || !sampleSize) st = gt::fail(GT_EINVAL, "null argument");
  else st = gt_kendall(X, *nx, Y, *ny, *sampleSize, answers);
  gt::report(st, "RgpuKendall");
}

void rBSplineMutualInfo(const int *nBins, const int *splineOrder, const int *nsamples,
                        const int *rowsA, const float *A, const int *rowsB, const float *B,
                        float *mutualInfo) {
  gt::clear_error();
  int st;
  if (!nBins || !splineOrder || !nsamples || !rowsA || !rowsB)
    st = gt::fail(GT_EINVAL, "null argument");
  else
    st = gt_mutual_info(*nBins, *splineOrder, *nsamples, A, *rowsA, B, *rowsB, mutualInfo);
  gt::report(st, "rBSplineMutualInfo");
}

// src/rinterface.cpp:216-239: the full n x n matrix of R's as.matrix(dist).
void Rhcluster(const float *distMat, const int *numPoints, int *merge, int *order, float *val,
               const char **method) {
  gt::clear_error();
  int st;
  if (!numPoints || !method) st = gt::fail(GT_EINVAL, "null argument");
  else st = gt_hclust(distMat, *numPoints, *method, merge, order, val);
  gt::report(st, "Rhcluster");
}

// src/rinterface.cpp:172-204: distances (p = 2) stay on the device.
void Rdistclust(const char **distmethod, const char **clustmethod, const float *points,
                const int *numPoints, const int *dim, int *merge, int *order, float *val) {
  gt::clear_error();
  int st;
  if (!distmethod || !clustmethod || !numPoints || !dim)
    st = gt::fail(GT_EINVAL, "null argument");
  else
    st = gt_distclust(points, *numPoints, *dim, gt::dist_enum(*distmethod), *clustmethod, merge,
                      order, val);
  gt::report(st, "Rdistclust");
}

// src/correlation.cpp:163-171 setDevice: ids outside [0, count) are an error.
void rsetDevice(const int *device) {
  gt::clear_error();
  int count = 0, st = GT_OK;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) {
    st = gt::fail(GT_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
  } else if (!device || *device < 0 || *device >= count) {
    st = gt::fail(GT_EINVAL, "The gpu id number is not valid.");
  } else {
    e = cudaSetDevice(*device);
    if (e != cudaSuccess) st = gt::fail(GT_ECUDA, "choosing gpu: %s", cudaGetErrorString(e));
  }
  gt::report(st, "rsetDevice");
}

void rgetDevice(int *device) {
  gt::clear_error();
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) {
    gt::report(gt::fail(GT_ENODEV, "no CUDA device: %s", cudaGetErrorString(e)), "rgetDevice");
    return;
  }
  if (device) *device = d;
}

void rtestT(const float *pairs, const float *coeffs, const int *n, float *ts) {
  gt::clear_error();
  int st = GT_OK;
  if (!n || *n < 0) {
    st = gt::fail(GT_EINVAL, "bad length");
  } else if (*n > 0) {
    const size_t b = size_t(*n) * 4;
    cudaStream_t s = gt::lib_stream();
    gt::StreamSyncGuard guard(s);
    void *dp = nullptr, *dc = nullptr, *dt = nullptr;
    st = gt::ws_get(gt::WS_IN_A, b, &dp);
    if (st == GT_OK) st = gt::ws_get(gt::WS_IN_B, b, &dc);
    if (st == GT_OK) st = gt::ws_get(gt::WS_OUT0, b, &dt);
    if (st == GT_OK) {
      cudaMemcpyAsync(dp, pairs, b, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dc, coeffs, b, cudaMemcpyHostToDevice, s);
      st = gt_ttest_device(static_cast<float *>(dp), static_cast<float *>(dc), *n,
                           static_cast<float *>(dt), s);
      if (st == GT_OK) {
        cudaMemcpyAsync(ts, dt, b, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = gt::fail(GT_ECUDA, "rtestT: %s", cudaGetErrorString(e));
      }
    }
  }
  gt::report(st, "rtestT");
}

// Host-buffer adjoints for the R gradient wrappers (no counterpart in the
// reference): copy in, run the device adjoint, copy out, synchronously.
void RgpuCorBackward(const float *X, const int *nobs, const int *nvar, const float *G,
                     float *dX) {
  gt::clear_error();
  int st = GT_OK;
  if (!nobs || !nvar || *nobs < 0 || *nvar < 0) {
    st = gt::fail(GT_EINVAL, "bad sizes");
  } else if (*nobs > 0 && *nvar > 0) {
    const int64_t n = *nobs, p = *nvar;
    const size_t bx = size_t(p) * size_t(n) * 4, bg = size_t(p) * size_t(p) * 4;
    cudaStream_t s = gt::lib_stream();
    gt::StreamSyncGuard guard(s);
    void *dx = nullptr, *dg = nullptr, *dout = nullptr;
    st = gt::ws_get(gt::WS_IN_A, bx, &dx);
    if (st == GT_OK) st = gt::ws_get(gt::WS_IN_B, bg, &dg);
    if (st == GT_OK) st = gt::ws_get(gt::WS_OUT0, bx, &dout);
    if (st == GT_OK) {
      cudaMemcpyAsync(dx, X, bx, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dg, G, bg, cudaMemcpyHostToDevice, s);
      st = gt_cor_backward_device(static_cast<float *>(dx), p, n, static_cast<float *>(dg),
                                  static_cast<float *>(dout), s);
      if (st == GT_OK) {
        cudaMemcpyAsync(dX, dout, bx, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = gt::fail(GT_ECUDA, "%s", cudaGetErrorString(e));
      }
    }
  }
  gt::report(st, "RgpuCorBackward");
}

void RgpuDistBackward(const float *points, const int *numPoints, const int *dim, const float *G,
                      float *dX) {
  gt::clear_error();
  int st = GT_OK;
  if (!numPoints || !dim || *numPoints < 0 || *dim < 0) {
    st = gt::fail(GT_EINVAL, "bad sizes");
  } else if (*numPoints > 0 && *dim > 0) {
    const int64_t n = *numPoints, d = *dim;
    const size_t bx = size_t(n) * size_t(d) * 4, bg = size_t(n) * size_t(n) * 4;
    cudaStream_t s = gt::lib_stream();
    gt::StreamSyncGuard guard(s);
    void *dx = nullptr, *dg = nullptr, *dout = nullptr;
    st = gt::ws_get(gt::WS_IN_A, bx, &dx);
    if (st == GT_OK) st = gt::ws_get(gt::WS_IN_B, bg, &dg);
    if (st == GT_OK) st = gt::ws_get(gt::WS_OUT0, bx, &dout);
    if (st == GT_OK) {
      cudaMemcpyAsync(dx, points, bx, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dg, G, bg, cudaMemcpyHostToDevice, s);
      st = gt_dist_backward_device(static_cast<float *>(dx), n, d, static_cast<float *>(dg),
                                   static_cast<float *>(dout), s);
      if (st == GT_OK) {
        cudaMemcpyAsync(dX, dout, bx, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = gt::fail(GT_ECUDA, "%s", cudaGetErrorString(e));
      }
    }
  }
  gt::report(st, "RgpuDistBackward");
}

void RgpuMdsStress(const float *points, const int *numPoints, const int *dim, const float *delta,
                   double *loss, float *dX) {
  gt::clear_error();
  int st = GT_OK;
  if (!numPoints || !dim || *numPoints < 0 || *dim < 0) {
    st = gt::fail(GT_EINVAL, "bad sizes");
  } else if (*numPoints > 0 && *dim > 0) {
    const int64_t n = *numPoints, d = *dim;
    const size_t bx = size_t(n) * size_t(d) * 4, bd = size_t(n) * size_t(n - 1) / 2 * 4;
    cudaStream_t s = gt::lib_stream();
    gt::StreamSyncGuard guard(s);
    void *dx = nullptr, *dd = nullptr, *dout = nullptr, *dl = nullptr;
    st = gt::ws_get(gt::WS_IN_A, bx, &dx);
    if (st == GT_OK) st = gt::ws_get(gt::WS_IN_B, bd > 0 ? bd : 4, &dd);
    if (st == GT_OK) st = gt::ws_get(gt::WS_OUT0, bx, &dout);
    if (st == GT_OK) st = gt::ws_get(gt::WS_OUT1, 8, &dl);
    if (st == GT_OK) {
      cudaMemcpyAsync(dx, points, bx, cudaMemcpyHostToDevice, s);
      if (bd) cudaMemcpyAsync(dd, delta, bd, cudaMemcpyHostToDevice, s);
      st = gt_mds_stress_device(static_cast<float *>(dx), n, d, static_cast<float *>(dd),
                                static_cast<float *>(dout), static_cast<double *>(dl), s);
      if (st == GT_OK) {
        if (dX) cudaMemcpyAsync(dX, dout, bx, cudaMemcpyDeviceToHost, s);
        if (loss) cudaMemcpyAsync(loss, dl, 8, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = gt::fail(GT_ECUDA, "%s", cudaGetErrorString(e));
      }
    }
  }
  gt::report(st, "RgpuMdsStress");
}

// The reference NVRTC-compiles inst/cuda/*.cu here (src/cudaUtils.cpp:118-165);
// this library ships sm_103a code, so loading only checks for a device.
void cuCompile(const int *numFiles, const char **cuFilenames, const char **cuSrc) {
  (void)numFiles; (void)cuFilenames; (void)cuSrc;
  gt::clear_error();
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    gt::report(gt::fail(GT_ENODEV, "no CUDA device available"), "cuCompile");
}

void unloadPackage(void) { gt::ws_release_all(); }

}  // extern "C"
