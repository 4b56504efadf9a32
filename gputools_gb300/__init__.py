"""gputools_gb300 -- GB300 (sm_103a) implementation of gputools' all-pairs
hot path: gpuDist (euclidean, maximum, manhattan, canberra, binary,
minkowski), gpuCor (pearson, kendall) and gpuMi (B-spline mutual
information).

The compute path is libgputools_gb300.so (hand-written CUDA for sm_103a) and
its C ABI, include/gputools_gb300.h; this package is the Python mirror of the
R API over that ABI.
"""
from .api import (BatchPlan, Dist, chooseGpu, distances_device, get_gram_path, getGpuId, gpuCor,
                  gpuCorBackward, gpuDist, gpuDistBackward, gpuMdsStress, gpuMi, gpuTtest,
                  kendall_device, mutual_info_device, pmcc_device, pmatch, set_gram_path)
from ._lib import GpuToolsError, load, last_error
from .builder import build

__all__ = ["BatchPlan", "Dist", "chooseGpu", "distances_device", "get_gram_path", "getGpuId", "gpuCor",
           "gpuCorBackward", "gpuDistBackward", "gpuMdsStress", "gpuDist", "gpuMi", "gpuTtest",
           "kendall_device", "mutual_info_device", "pmcc_device", "pmatch", "set_gram_path",
           "GpuToolsError", "load", "last_error", "build"]
