// Link-time pieces of the oracle's build of the reference's GPU path
// (test infrastructure, never shipped): R's error reporting, the by-name
// launcher the reference's host code calls (src/cudaUtils.h cudaLaunch), its
// CUDA error check (src/cuseful.cpp:95-102), and plain C entry points into
// the reference's host functions, so that a test script can call pmcc(),
// bSplineMutualInfo(), hcluster(), distance() and masterKendall() on a GPU
// and record what the reference itself returns.
//
// The launcher runs each kernel with cudaLaunchKernel from the registry of
// ahead-of-time compiled kernels, instead of loading and unloading an NVRTC
// module around every launch as src/cudaUtils.cpp:197-218 does; the kernels,
// their arguments, grids and the host orchestration are the reference's.
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

#include <cuda_runtime_api.h>

#include "gpu_registry.h"

#include "correlation.h"
#include "distance.h"
#include "hcluster.h"
#include "kendall.h"
#include "mi.h"

std::map<std::string, const void *> &ref_kernel_table() {
  static std::map<std::string, const void *> t;
  return t;
}

extern "C" void error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::fprintf(stderr, "reference error: ");
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fprintf(stderr, "\n");
  std::abort();
}
extern "C" void warning(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fprintf(stderr, "\n");
}
extern "C" void Rprintf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vprintf(fmt, ap);
  va_end(ap);
}

void cudaLaunch(std::string kernelName, void *args[], const dim3 &gridDim, const dim3 &blockDim,
                cudaStream_t stream) {
  auto &t = ref_kernel_table();
  auto it = t.find(kernelName);
  if (it == t.end()) error("kernel %s is not in the registry", kernelName.c_str());
  cudaError_t e = cudaLaunchKernel(it->second, gridDim, blockDim, args, 0, stream);
  if (e != cudaSuccess) error("launch of %s: %s", kernelName.c_str(), cudaGetErrorString(e));
}

void fatal(const char *msg) { error("%s", msg); }
void checkCudaError(const char *msg) {
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) error("%s: %s", msg ? msg : "", cudaGetErrorString(err));
}
void checkCublasError(const char *msg) { (void)msg; }

extern "C" {

// rpmcc (src/rinterface.cpp:33-55) without the R layer: whichObs 0 =
// everything, 1 = pairwise.complete.obs.
int ref_pmcc(int use, const float *A, size_t na, const float *B, size_t nb, size_t n,
             float *pairs, float *corr, float *ts) {
  pmcc(use == 0 ? everything : pairwiseComplete, A, na, B, nb, n, pairs, corr, ts);
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : int(e);
}

// rBSplineMutualInfo (src/rinterface.cpp:415-422) without the R layer.
int ref_mi(int nbins, int order, int nsamples, int nx, const float *x, int ny, const float *y,
           float *out) {
  bSplineMutualInfo(nbins, order, nsamples, nx, x, ny, y, out);
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : int(e);
}

// Rhcluster's call of hcluster (src/rinterface.cpp:216-239), returning the
// step list (sub, sup, heights) before formatClustering.
int ref_hcluster(const float *dist, size_t n, int method, int *sub, int *sup, float *val) {
  hcluster(dist, n * sizeof(float), n, sub, sup, val, hc_method(method), 0.5f, 0.5f);
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : int(e);
}

// Rdistances (src/rinterface.cpp:206-214) without the R layer.
int ref_distance(const float *points, size_t n, size_t dim, float *out, int method, float p) {
  distance(points, dim * sizeof(float), n, points, dim * sizeof(float), n, dim, out,
           n * sizeof(float), dist_method(method), p);
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : int(e);
}

// RgpuKendall (src/rinterface.cpp:128-132) without the R layer.
int ref_kendall(const float *x, size_t nx, const float *y, size_t ny, size_t n, double *out) {
  masterKendall(x, nx, y, ny, n, out);
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : int(e);
}

}  // extern "C"
