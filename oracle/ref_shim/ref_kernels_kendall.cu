// The reference's Kendall kernel (inst/cuda/kendall.cu), registered by name.
// Test infrastructure only.
#include "kendall.cu"
#include "gpu_registry.h"
REF_KERNEL(gpuKendall)
