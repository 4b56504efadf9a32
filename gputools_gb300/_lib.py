"""ctypes binding of libgputools_gb300.so (the C ABI in include/gputools_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises, it never falls back to a CPU or PyTorch implementation.
"""
from __future__ import annotations

import ctypes
import os

from . import builder as _build

LIB_PATH = _build.LIB

GT_OK = 0
GT_EINVAL = 1
GT_ECUDA = 2
GT_ENOMEM = 3
GT_ENODEV = 4
GT_ETIMEOUT = 5
GT_EUNSUPPORTED = 6

GT_LAYOUT_FULL = 0
GT_LAYOUT_DIST = 1

GT_GRAM_TC_BF16X3 = 0
GT_GRAM_TC_BF16X6 = 1
GT_GRAM_FP32 = 2
GT_GRAM_TC_F16X3 = 3
GT_GRAM_TC_F16X6 = 4

# (name, restype, argtypes) of every symbol include/gputools_gb300.h declares.
_i, _i64, _f, _vp, _cp = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p, ctypes.c_char_p
_pi = ctypes.POINTER(ctypes.c_int)
_pf = ctypes.POINTER(ctypes.c_float)
_pcp = ctypes.POINTER(ctypes.c_char_p)
SIGNATURES = {
    # .C entry points of the reference
    "Rdistances": (None, [_vp, _pi, _pi, _vp, _pcp, _pf]),
    "rpmcc": (None, [_pi, _vp, _pi, _vp, _pi, _pi, _vp, _vp, _vp]),
    "RgpuKendall": (None, [_vp, _pi, _vp, _pi, _pi, _vp]),
    "rBSplineMutualInfo": (None, [_pi, _pi, _pi, _pi, _vp, _pi, _vp, _vp]),
    "Rhcluster": (None, [_vp, _pi, _vp, _vp, _vp, _pcp]),
    "Rdistclust": (None, [_pcp, _pcp, _vp, _pi, _pi, _vp, _vp, _vp]),
    "rsetDevice": (None, [_pi]),
    "rgetDevice": (None, [_pi]),
    "rtestT": (None, [_vp, _vp, _pi, _vp]),
    "cuCompile": (None, [_pi, _pcp, _pcp]),
    "unloadPackage": (None, []),
    # status API
    "gt_last_error": (_cp, []),
    "gt_version": (_i, []),
    "gt_release_workspace": (None, []),
    "gt_device_status": (_i, [_vp]),
    "gt_set_wait_limit_ns": (_i, [ctypes.c_uint64]),
    "gt_kernel_launches": (ctypes.c_uint64, []),
    "gt_profile_enable": (None, [_i]),
    "gt_profile_reset": (None, []),
    "gt_profile_kernel_ms": (_i, [_cp, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_uint64)]),
    "gt_set_gram_path": (_i, [_i]),
    "gt_get_gram_path": (_i, []),
    "gt_distances": (_i, [_vp, _i64, _i64, _vp, _i, _f]),
    "gt_distances_device": (_i, [_vp, _i64, _i64, _vp, _i, _i, _f, _vp]),
    "gt_pmcc": (_i, [_i, _vp, _i64, _vp, _i64, _i64, _vp, _vp, _vp]),
    "gt_pmcc_device": (_i, [_i, _vp, _i64, _vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gt_pmcc_device_noalloc": (_i, [_i, _vp, _i64, _vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    "gt_kendall": (_i, [_vp, _i64, _vp, _i64, _i64, _vp]),
    "gt_kendall_device": (_i, [_vp, _i64, _vp, _i64, _i64, _vp, _vp]),
    "gt_mutual_info": (_i, [_i, _i, _i64, _vp, _i64, _vp, _i64, _vp]),
    "gt_mutual_info_device": (_i, [_i, _i, _i64, _vp, _i64, _vp, _i64, _vp, _vp]),
    "gt_hclust": (_i, [_vp, _i64, _cp, _vp, _vp, _vp]),
    "gt_hclust_device": (_i, [_vp, _i64, _cp, _vp, _vp, _vp, _vp]),
    "gt_distclust": (_i, [_vp, _i64, _i64, _i, _cp, _vp, _vp, _vp]),
    "gt_hclust_format": (_i, [_i, _vp, _vp, _vp, _vp]),
    "gt_ttest_device": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "gt_cor_backward_device": (_i, [_vp, _i64, _i64, _vp, _vp, _vp]),
    "gt_dist_backward_device": (_i, [_vp, _i64, _i64, _vp, _vp, _vp]),
    "gt_mds_stress_device": (_i, [_vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    "RgpuCorBackward": (None, [_vp, _pi, _pi, _vp, _vp]),
    "RgpuDistBackward": (None, [_vp, _pi, _pi, _vp, _vp]),
    "RgpuMdsStress": (None, [_vp, _pi, _pi, _vp, _vp, _vp]),
}

class CorProblem(ctypes.Structure):
    """gt_cor_problem: one cor(x) of a batch (device pointers)."""
    _fields_ = [("X", ctypes.c_void_p), ("p", ctypes.c_int64), ("n", ctypes.c_int64),
                ("corr", ctypes.c_void_p), ("ts", ctypes.c_void_p), ("pairs", ctypes.c_void_p),
                ("ld", ctypes.c_int64)]


class KendallProblem(ctypes.Structure):
    """gt_kendall_problem: one Kendall cor(x) of a batch (device pointers)."""
    _fields_ = [("X", ctypes.c_void_p), ("p", ctypes.c_int64), ("n", ctypes.c_int64),
                ("out", ctypes.c_void_p)]


GT_BATCH_NO_GRAPH = 1
GT_BATCH_AUTOTUNE = 2

SIGNATURES.update({
    "gt_pmcc_batch_plan_create": (_i, [ctypes.POINTER(CorProblem), _i64, _i,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "gt_kendall_batch_plan_create": (_i, [ctypes.POINTER(KendallProblem), _i64, _i,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "gt_batch_plan_launch": (_i, [_vp, _vp]),
    "gt_batch_plan_describe": (_cp, [_vp]),
    "gt_batch_plan_destroy": (None, [_vp]),
})

_lib = None


class GpuToolsError(RuntimeError):
    """A gt_* call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def load(path: str = LIB_PATH):
    """Load the shared library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libgputools_gb300.so not found at {path}")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().gt_last_error()
    return msg.decode() if msg else ""


def check(status: int) -> None:
    if status != GT_OK:
        raise GpuToolsError(status, last_error())
