// Link-time stand-ins for the parts of the reference that the CPU loops do
// not use (R's error reporting, the NVRTC kernel launcher in
// src/cudaUtils.cpp, the error helpers in src/cuseful.cpp).  Calling any GPU
// entry of the reference through this build is an error by design: only the
// CPU functions distance_host, hostKendall, permHostKendall and hostSignif
// are exercised.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <cuda_runtime_api.h>

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
}
extern "C" void Rprintf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vprintf(fmt, ap);
  va_end(ap);
}
void cudaLaunch(std::string kernelName, void *args[], const dim3 &, const dim3 &,
                cudaStream_t) {
  (void)args;
  error("GPU launch of %s is not part of the CPU reference build", kernelName.c_str());
}
void fatal(const char *msg) { error("%s", msg); }
void checkCudaError(const char *msg) { (void)msg; }
void checkCublasError(const char *msg) { (void)msg; }
