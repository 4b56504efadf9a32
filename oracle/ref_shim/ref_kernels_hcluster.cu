// The reference's clustering kernels (inst/cuda/hcluster.cu), registered by
// name.  Test infrastructure only.  CUDART_INF_F comes from
// math_constants.h (force-included by the build recipe).
#include "hcluster.cu"
#include "gpu_registry.h"
REF_KERNEL(convert_kernel)
REF_KERNEL(find_min1_kernel)
REF_KERNEL(find_min2_kernel)
REF_KERNEL(single_kernel)
REF_KERNEL(complete_kernel)
REF_KERNEL(wpgma_kernel)
REF_KERNEL(average_kernel)
REF_KERNEL(median_kernel)
REF_KERNEL(centroid_kernel)
REF_KERNEL(flexible_group_kernel)
REF_KERNEL(flexible_kernel)
REF_KERNEL(ward_kernel)
REF_KERNEL(mcquitty_kernel)
