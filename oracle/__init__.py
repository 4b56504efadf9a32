"""FP64 CPU oracle for gputools' all-pairs statistics.

TEST INFRASTRUCTURE ONLY.  Only tests/, bench.py's CPU-baseline leg (and its
``--impl reference`` arm) and ``__graft_entry__.smoke()`` may import this
package, and only as the checker or the CPU baseline.  The shipped library
(`gputools_gb300`) never imports, links or calls it.

Two back ends:

* ``liboracle.so`` -- ``oracle.c``, a double-precision restatement of R's
  ``stats::dist`` / ``stats::cor`` semantics as gputools exposes them (see
  ``oracle.h`` for the reference lines each function follows).
* ``_ref/libref_cpu.so`` -- the reference's own CPU loops compiled straight
  from the reference tree by ``build_ref.sh`` (``distance_host`` in
  src/distance.cpp:174-207, ``hostKendall``/``permHostKendall`` in
  src/correlation.cpp:488-516, ``hostSignif`` in src/correlation.cpp:51-64).
  It pins the restatement (tests/test_oracle.py) and generated
  tests/golden/reference_cpu.npz; on the GPU hosts it is built from the
  staged copy and timed as the reference's host loops.
* ``baseline/_ref/libref_gpu.so`` -- the reference's own GPU path (host
  orchestration in src/*.cpp, kernels in inst/cuda/*.cu) built by
  ``build_ref_gpu.sh`` from a copy that ``stage_ref.sh`` places in the
  git-ignored baseline/_ref/ (the GPU hosts receive it, the reference tree
  itself is absent there).  tests/golden/make_golden_gpu.py runs it on a GPU
  to record tests/golden/reference_gpu.npz, which pins the restatement of
  Pearson, gpuMi and the clustering to what the reference itself returns.

Parity pinning: the reference ships no tests or golden vectors, so the oracle
is pinned (a) against the reference's own CPU loops (float32 arithmetic, so to
float32 tolerance) and the committed fixtures made from them, and (b) against
scipy / numpy implementations of the same R definitions.  R itself is not
available, so R's last-bit behaviour (Kendall tau-b evaluation order) is
restated, not run.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_cpu.so")
STAGED = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "gputools")
REF_GPU_LIB = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "libref_gpu.so")

METHODS = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")

_lib = None
_ref = None


def reference_root(staged: bool = True) -> Optional[str]:
    """Where the reference source tree is: $GPUTOOLS_REFERENCE, else the
    ``reference_path`` recorded in the repository's benchmark spec, else (with
    ``staged``) the copy stage_ref.sh left in baseline/_ref/gputools; None
    when none of them exists."""
    root = os.environ.get("GPUTOOLS_REFERENCE")
    if not root:
        try:
            import json
            with open(os.path.join(os.path.dirname(HERE), "BASELINE.json")) as f:
                root = json.load(f).get("reference_path")
        except (OSError, ValueError):
            root = None
    if root and os.path.isfile(os.path.join(root, "src", "correlation.cpp")):
        return root
    if staged and os.path.isfile(os.path.join(STAGED, "src", "correlation.cpp")):
        return STAGED
    return None


def build(force: bool = False) -> str:
    """Compile oracle.c (gcc, -O3, OpenMP) into _build/liboracle.so, and the
    reference CPU loops into _ref/ when the reference tree is present."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        subprocess.check_call(
            ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-Wall", "-ffp-contract=off",
             "-o", LIB, src, "-lm"])
    ref_script = os.path.join(HERE, "build_ref.sh")
    real = reference_root(staged=False)
    if real and os.path.realpath(real) != os.path.realpath(STAGED):
        # copy the hot path's sources where the GPU hosts receive them
        subprocess.check_call(["bash", os.path.join(HERE, "stage_ref.sh"), real],
                              stdout=subprocess.DEVNULL)
    ref = reference_root()
    if (force or not os.path.exists(REF_LIB)) and ref:
        subprocess.check_call(["bash", ref_script], env=dict(os.environ, GPUTOOLS_REFERENCE=ref))
    if (force or not os.path.exists(REF_GPU_LIB)) and os.path.isdir(STAGED):
        subprocess.check_call(["bash", os.path.join(HERE, "build_ref_gpu.sh"), STAGED])
    return LIB


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        i64, dp, fp = ctypes.c_int64, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
        lib.orc_dist.argtypes = [fp, i64, fp, i64, i64, ctypes.c_int, ctypes.c_double, fp]
        lib.orc_pearson.argtypes = [ctypes.c_int, fp, i64, fp, i64, i64, fp, fp, fp]
        lib.orc_kendall.argtypes = [fp, i64, fp, i64, i64, ctypes.c_int, fp, fp, fp, fp]
        lib.orc_ttest.argtypes = [fp, fp, i64, fp]
        lib.orc_signif.argtypes = [fp, fp, i64, fp]
        lib.orc_cor_backward.argtypes = [fp, i64, i64, fp, fp]
        lib.orc_dist_backward.argtypes = [fp, i64, i64, fp, fp]
        lib.orc_mds_stress.argtypes = [fp, i64, i64, fp, fp, fp]
        lib.orc_bspline_mi.argtypes = [ctypes.c_int, ctypes.c_int, i64, fp, i64, fp, i64, fp, fp, fp]
        lib.orc_hc_method.argtypes = [ctypes.c_char_p]
        lib.orc_hclust.argtypes = [fp, i64, ctypes.c_int, ctypes.c_float, ctypes.c_float, fp, fp, fp]
        lib.orc_format_clustering.argtypes = [ctypes.c_int, fp, fp, fp, fp]
        lib.orc_set_threads.argtypes = [ctypes.c_int]
        lib.orc_get_threads.restype = ctypes.c_int
        del dp
        _lib = lib
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_gpu_available() -> bool:
    return os.path.exists(REF_GPU_LIB)


_ref_gpu = None


def _ref_gpu_lib():
    """The reference's GPU path (needs a CUDA device to call)."""
    global _ref_gpu
    if _ref_gpu is None:
        if not ref_gpu_available():
            raise RuntimeError("reference GPU build missing: run oracle/build_ref_gpu.sh on a "
                               "host with the staged reference tree")
        lib = ctypes.CDLL(REF_GPU_LIB)
        sz, fp, ci = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        lib.ref_pmcc.argtypes = [ci, fp, sz, fp, sz, sz, fp, fp, fp]
        lib.ref_mi.argtypes = [ci, ci, ci, ci, fp, ci, fp, fp]
        lib.ref_hcluster.argtypes = [fp, sz, ci, fp, fp, fp]
        lib.ref_distance.argtypes = [fp, sz, sz, fp, ci, ctypes.c_float]
        lib.ref_kendall.argtypes = [fp, sz, fp, sz, sz, fp]
        _ref_gpu = lib
    return _ref_gpu


def _check_ref(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"reference {what} failed (CUDA error {rc})")


def ref_gpu_pmcc(A: np.ndarray, B: np.ndarray, use: int = 0):
    """The reference's pmcc() (src/correlation.cpp:66-161) on the GPU: A
    (na, n), B (nb, n) variable-major, passed as two buffers as R's .C does.
    Returns (corr, pairs, ts), float32 (na, nb)."""
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    na, n = A.shape
    nb = B.shape[0]
    corr = np.empty((na, nb), np.float32); pairs = np.empty_like(corr); ts = np.empty_like(corr)
    _check_ref(_ref_gpu_lib().ref_pmcc(int(use), _ptr(A), na, _ptr(B), nb, n, _ptr(pairs),
                                       _ptr(corr), _ptr(ts)), "pmcc")
    return corr, pairs, ts


def ref_gpu_mi(X: np.ndarray, bins: int, order: int) -> np.ndarray:
    """The reference's bSplineMutualInfo (src/mi.cpp:33-164) of X with itself
    (the reference kernel get_mi is only in bounds for nx == ny).  X (nx, n)
    variable-major; returns out[y, x] (nx, nx) float32."""
    X = np.ascontiguousarray(X, np.float32)
    nx, n = X.shape
    out = np.empty((nx, nx), np.float32)
    _check_ref(_ref_gpu_lib().ref_mi(int(bins), int(order), n, nx, _ptr(X), nx, _ptr(X),
                                     _ptr(out)), "bSplineMutualInfo")
    return out


def ref_gpu_hcluster(D: np.ndarray, method: str):
    """The reference's hcluster (src/hcluster.cpp:15-38) on the full n x n
    float matrix D; returns the step list (sub, sup, heights)."""
    D = np.ascontiguousarray(D, np.float32)
    n = D.shape[0]
    sub = np.empty(n - 1, np.int32); sup = np.empty(n - 1, np.int32)
    val = np.empty(n - 1, np.float32)
    code = _load().orc_hc_method(method.encode())
    _check_ref(_ref_gpu_lib().ref_hcluster(_ptr(D), n, int(code), _ptr(sub), _ptr(sup),
                                           _ptr(val)), "hcluster")
    return sub, sup, val


def ref_gpu_distance(P: np.ndarray, method: str, p: float = 2.0) -> np.ndarray:
    """The reference's distance() (src/distance.cpp:259-316) of the rows of
    P with themselves; returns the full (n, n) float32 matrix."""
    P = np.ascontiguousarray(P, np.float32)
    n, dim = P.shape
    out = np.empty((n, n), np.float32)
    _check_ref(_ref_gpu_lib().ref_distance(_ptr(P), n, dim, _ptr(out), method_index(method),
                                           float(p)), "distance")
    return out


def ref_gpu_kendall(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """The reference's masterKendall (src/kendall.cpp:13-55): out[y, x]."""
    X = np.ascontiguousarray(X, np.float32); Y = np.ascontiguousarray(Y, np.float32)
    nx, n = X.shape
    ny = Y.shape[0]
    out = np.empty((ny, nx), np.float64)
    _check_ref(_ref_gpu_lib().ref_kendall(_ptr(X), nx, _ptr(Y), ny, n, _ptr(out)), "kendall")
    return out


def _ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference CPU build missing: run oracle/build_ref.sh "
                               "where the reference tree is present")
        _ref = ctypes.CDLL(REF_LIB)
    return _ref


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    _load().orc_set_threads(int(n))


def threads() -> int:
    return int(_load().orc_get_threads())


def method_index(method: str) -> int:
    return METHODS.index(method)


def dist(a: np.ndarray, method: str = "euclidean", p: float = 2.0,
         b: Optional[np.ndarray] = None) -> np.ndarray:
    """Distances between the rows of ``a`` (and ``b``; default ``a``).

    Returns D with D[y, x] = d(a_x, b_y), float64 (the reference layout
    d[y*N + x])."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a if b is None else np.ascontiguousarray(b, dtype=np.float32)
    if a.ndim != 2 or b.ndim != 2 or a.shape[1] != b.shape[1]:
        raise ValueError("points must be 2-D with equal dimension")
    out = np.empty((b.shape[0], a.shape[0]), dtype=np.float64)
    rc = _load().orc_dist(_ptr(a), a.shape[0], _ptr(b), b.shape[0], a.shape[1],
                          method_index(method), float(p), _ptr(out))
    if rc != 0:
        raise ValueError(f"orc_dist failed ({rc})")
    return out


def pearson(A: np.ndarray, B: Optional[np.ndarray] = None, use: int = 0):
    """Pearson r for every pair of variables.

    ``A`` is (na, n): one variable per row, observations contiguous (the
    reference's A[x*n + k]).  Returns (corr, pairs, ts), each (na, nb) with
    [x, y] the pair (A_x, B_y)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = A if B is None else np.ascontiguousarray(B, dtype=np.float32)
    na, n = A.shape
    nb = B.shape[0]
    if B.shape[1] != n:
        raise ValueError("A and B need the same number of observations")
    corr = np.empty((na, nb)); pairs = np.empty((na, nb)); ts = np.empty((na, nb))
    rc = _load().orc_pearson(int(use), _ptr(A), na, _ptr(B), nb, n, _ptr(corr),
                             _ptr(pairs), _ptr(ts))
    if rc != 0:
        raise ValueError(f"orc_pearson failed ({rc})")
    return corr, pairs, ts


def kendall(X: np.ndarray, Y: Optional[np.ndarray] = None, same: Optional[bool] = None):
    """Kendall tau-b for every pair of variables; X is (nx, n), Y (ny, n).

    Returns (tau, S, Tx, Ty), each shaped (ny, nx) -- the reference's
    results[y*nx + x] layout."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    if same is None:
        same = Y is None
    Y = X if Y is None else np.ascontiguousarray(Y, dtype=np.float32)
    nx, n = X.shape
    ny = Y.shape[0]
    tau = np.empty((ny, nx)); S = np.empty((ny, nx), np.int64)
    Tx = np.empty((ny, nx), np.int64); Ty = np.empty((ny, nx), np.int64)
    rc = _load().orc_kendall(_ptr(X), nx, _ptr(Y), ny, n, int(bool(same)), _ptr(tau),
                             _ptr(S), _ptr(Tx), _ptr(Ty))
    if rc != 0:
        raise ValueError(f"orc_kendall failed ({rc})")
    return tau, S, Tx, Ty


def ttest(pairs: np.ndarray, r: np.ndarray) -> np.ndarray:
    pairs = np.ascontiguousarray(pairs, np.float64); r = np.ascontiguousarray(r, np.float64)
    out = np.empty_like(r)
    _load().orc_ttest(_ptr(pairs), _ptr(r), r.size, _ptr(out))
    return out


def signif(pairs: np.ndarray, r: np.ndarray) -> np.ndarray:
    pairs = np.ascontiguousarray(pairs, np.float64); r = np.ascontiguousarray(r, np.float64)
    out = np.empty_like(r)
    _load().orc_signif(_ptr(pairs), _ptr(r), r.size, _ptr(out))
    return out


# ---------------------------------------------------------------------------
# The reference's own CPU loops (float32), for pinning the restatement.

def ref_distance_host(points: np.ndarray, method: str = "euclidean", p: float = 2.0) -> np.ndarray:
    """src/distance.cpp:174-207 ``distance_host`` on the rows of ``points``.

    That function writes d[y*dim + x] (its row stride is the dimension, not
    n_a), so it is called once per y with n_b = 1, where the stride is
    irrelevant.  Returns (N, N) float32 with [y, x] = d(x, y)."""
    lib = _ref_lib()
    fn = lib._Z13distance_hostPKfmmS0_mmmPfm11dist_methodf
    sz = ctypes.c_size_t
    fn.argtypes = [ctypes.c_void_p, sz, sz, ctypes.c_void_p, sz, sz, sz, ctypes.c_void_p,
                   sz, ctypes.c_int, ctypes.c_float]
    pts = np.ascontiguousarray(points, np.float32)
    N, D = pts.shape
    out = np.empty((N, N), np.float32)
    row = np.empty(max(N, D), np.float32)
    for y in range(N):
        fn(_ptr(pts), D * 4, N, pts[y:y + 1].ctypes.data_as(ctypes.c_void_p), D * 4, 1, D,
           _ptr(row), N * 4, method_index(method), float(p))
        out[y] = row[:N]
    return out


def ref_host_kendall(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """src/correlation.cpp:506-516 ``permHostKendall`` (the reference's tau-a
    variant, float counters).  Returns (ny, nx) with [y, x]."""
    lib = _ref_lib()
    fn = lib._Z15permHostKendallPKfmS0_mmPd
    sz = ctypes.c_size_t
    fn.argtypes = [ctypes.c_void_p, sz, ctypes.c_void_p, sz, sz, ctypes.c_void_p]
    X = np.ascontiguousarray(X, np.float32); Y = np.ascontiguousarray(Y, np.float32)
    nx, n = X.shape
    ny = Y.shape[0]
    out = np.empty((ny, nx), np.float64)
    fn(_ptr(X), nx, _ptr(Y), ny, n, _ptr(out))
    return out


def ref_host_signif(pairs: np.ndarray, r: np.ndarray) -> np.ndarray:
    """src/correlation.cpp:51-64 ``hostSignif`` (float32)."""
    lib = _ref_lib()
    fn = lib._Z10hostSignifPKfS0_mPf
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    pairs = np.ascontiguousarray(pairs, np.float32); r = np.ascontiguousarray(r, np.float32)
    out = np.empty(r.shape, np.float32)
    fn(_ptr(pairs), _ptr(r), r.size, _ptr(out))
    return out


# ---------------------------------------------------------------------------
# Adjoints (FP64), for the backward kernels.

def cor_backward(X: np.ndarray, G: np.ndarray) -> np.ndarray:
    """dL/dX for C = cor(X) (X variable-major (p, n)) given G = dL/dC (p, p)."""
    X = np.ascontiguousarray(X, np.float32)
    G = np.ascontiguousarray(G, np.float64)
    p, n = X.shape
    out = np.empty((p, n), np.float64)
    rc = _load().orc_cor_backward(_ptr(X), p, n, _ptr(G), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"orc_cor_backward failed ({rc})")
    return out


def dist_backward(X: np.ndarray, G: np.ndarray) -> np.ndarray:
    """dL/dX for D = euclidean distances of the rows of X given G = dL/dD."""
    X = np.ascontiguousarray(X, np.float32)
    G = np.ascontiguousarray(G, np.float64)
    n, d = X.shape
    out = np.empty((n, d), np.float64)
    _load().orc_dist_backward(_ptr(X), n, d, _ptr(G), _ptr(out))
    return out


def mds_stress(X: np.ndarray, delta: np.ndarray):
    """(loss, dL/dX) of sum_{i<j} (D_ij - delta_ij)^2, delta in R dist layout."""
    X = np.ascontiguousarray(X, np.float32)
    delta = np.ascontiguousarray(delta, np.float32)
    n, d = X.shape
    loss = np.zeros(1, np.float64)
    out = np.empty((n, d), np.float64)
    _load().orc_mds_stress(_ptr(X), n, d, _ptr(delta), _ptr(loss), _ptr(out))
    return float(loss[0]), out


def bspline_mi(X: np.ndarray, Y: Optional[np.ndarray] = None, bins: int = 2, order: int = 1):
    """B-spline mutual information (R's gpuMi): X (nx, n) and Y (ny, n), one
    variable per row.  Returns (mi, hx, hy) with mi[y, x] = MI(X_x, Y_y) (the
    reference layout out[y*nx + x]) and the entropies."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = X if Y is None else np.ascontiguousarray(Y, dtype=np.float32)
    nx, n = X.shape
    ny = Y.shape[0]
    out = np.empty((ny, nx), np.float64)
    hx = np.empty(nx, np.float64)
    hy = np.empty(ny, np.float64)
    rc = _load().orc_bspline_mi(int(bins), int(order), n, _ptr(X), nx, _ptr(Y), ny, _ptr(out),
                                _ptr(hx), _ptr(hy))
    if rc != 0:
        raise ValueError(f"orc_bspline_mi failed ({rc})")
    return out, hx, hy


def hclust(D: np.ndarray, method: str = "complete"):
    """Hierarchical clustering of the full (n, n) float32 distance matrix as
    the reference's kernels do it (gpuHclust).  Returns (sub, sup, height):
    per step the merged column and row indices and the merge height."""
    D = np.ascontiguousarray(D, dtype=np.float32)
    n = D.shape[0]
    sub = np.empty(n - 1, np.int32)
    sup = np.empty(n - 1, np.int32)
    val = np.empty(n - 1, np.float32)
    m = _load().orc_hc_method(method.encode())
    rc = _load().orc_hclust(_ptr(D), n, m, 0.5, 0.5, _ptr(sub), _ptr(sup), _ptr(val))
    if rc != 0:
        raise ValueError(f"orc_hclust failed ({rc})")
    return sub, sup, val


def format_clustering(sub: np.ndarray, sup: np.ndarray):
    """R's merge matrix ((n-1) x 2) and order (1-based) from sub/sup, as the
    reference's formatClustering does it."""
    sub = np.ascontiguousarray(sub, np.int32)
    sup = np.ascontiguousarray(sup, np.int32)
    ln = sub.size
    merge = np.empty(2 * ln, np.int32)
    order = np.empty(ln + 1, np.int32)
    _load().orc_format_clustering(ln, _ptr(sub), _ptr(sup), _ptr(merge), _ptr(order))
    return merge.reshape(2, ln).T.copy(), order
