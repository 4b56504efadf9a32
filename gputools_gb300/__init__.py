"""gputools_gb300 -- GB300 (sm_103a) implementation of gputools' all-pairs
hot path: gpuDist (euclidean, maximum, manhattan, canberra, binary,
minkowski), gpuCor (pearson, kendall), gpuMi (B-spline mutual information)
and gpuHclust / gpuDistClust (hierarchical clustering of those distances).

The compute path is libgputools_gb300.so (hand-written CUDA for sm_103a) and
its C ABI, include/gputools_gb300.h; this package is the Python mirror of the
R API over that ABI.
"""
from .api import (BatchPlan, Dist, HClust, chooseGpu, distances_device, get_gram_path, getGpuId,
                  gpuCor, gpuCorBackward, gpuDist, gpuDistBackward, gpuDistClust, gpuHclust,
                  gpuMdsStress, gpuMi, gpuTtest, hclust_device, hclust_format, kendall_device,
                  mutual_info_device, pmcc_device, pmatch, set_gram_path)
from ._lib import GpuToolsError, load, last_error
from .builder import build

__all__ = ["BatchPlan", "Dist", "HClust", "chooseGpu", "distances_device", "get_gram_path",
           "getGpuId", "gpuCor", "gpuCorBackward", "gpuDistBackward", "gpuDistClust", "gpuHclust",
           "gpuMdsStress", "gpuDist", "gpuMi", "gpuTtest", "hclust_device", "hclust_format",
           "kendall_device", "mutual_info_device", "pmcc_device", "pmatch", "set_gram_path",
           "GpuToolsError", "load", "last_error", "build"]
