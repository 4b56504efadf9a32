/* Force-included when compiling the reference's host files against CUDA 13,
 * which removed cudaThreadSynchronize (the reference calls it between
 * launches in src/correlation.cpp:128-140). */
#include <cuda_runtime_api.h>
#define cudaThreadSynchronize cudaDeviceSynchronize
