// The reference's distance kernels (inst/cuda/distance.cu), registered by
// name.  Test infrastructure only.
#include "distance.cu"
#include "gpu_registry.h"
REF_KERNEL(euclidean_kernel_same)
REF_KERNEL(maximum_kernel_same)
REF_KERNEL(manhattan_kernel_same)
REF_KERNEL(canberra_kernel_same)
REF_KERNEL(binary_kernel_same)
REF_KERNEL(minkowski_kernel_same)
