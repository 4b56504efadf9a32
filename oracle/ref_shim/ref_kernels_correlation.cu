// The reference's Pearson kernels (inst/cuda/correlation.cu), registered by
// name.  Test infrastructure only.
#include "correlation.cu"
#include "gpu_registry.h"
REF_KERNEL(gpuMeans)
REF_KERNEL(gpuSD)
REF_KERNEL(gpuPMCC)
REF_KERNEL(gpuMeansNoTest)
REF_KERNEL(gpuSDNoTest)
REF_KERNEL(gpuPMCCNoTest)
