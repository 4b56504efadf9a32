// The reference's B-spline mutual-information kernels (inst/cuda/mi.cu),
// registered by name.  Test infrastructure only.
#include "mi.cu"
#include "gpu_registry.h"
REF_KERNEL(scale)
REF_KERNEL(get_bin_scores)
REF_KERNEL(get_entropy)
REF_KERNEL(get_mi)
