"""Python mirror of gputools' R API for the all-pairs path.

Same function names, argument meanings, method matching and error messages
as the reference's R wrappers:

* ``gpuDist``  -- R/gpuHclust.R:1-39
* ``gpuCor``   -- R/gpuCor.R:1-62
* ``gpuTtest`` -- R/gpuCor.R:64-74
* ``chooseGpu`` / ``getGpuId`` -- R/chooseGpu.R, R/getGpuId.R

Matrices follow R's conventions: ``points`` is N x D with one point per row,
``x``/``y`` are n x p with one variable per column.  Results are float64
arrays, as R hands back the float32 outputs of ``.C`` as doubles.  Every
computation runs in libgputools_gb300.so through its C ABI.
"""
from __future__ import annotations

import ctypes
import warnings
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GT_LAYOUT_DIST, GT_LAYOUT_FULL, check, load

DIST_METHODS = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")
COR_METHODS = ("pearson", "kendall")
# R/gpuHclust.R gpuHclust's table; the chosen name goes to the library as is
# ("flexible group" is then single linkage, as in the reference).
HCLUST_METHODS = ("ward", "single", "complete", "average", "mcquitty", "median", "centroid",
                  "flexible", "flexible group", "wpgma")
COR_USES = ("everything", "pairwise.complete.obs")


def pmatch(x: str, table: Sequence[str]) -> Optional[int]:
    """R's pmatch for one string: exact match, else a unique prefix match,
    else None (no match or ambiguous; the empty string matches nothing)."""
    if not isinstance(x, str) or x == "":
        return None
    for i, t in enumerate(table):
        if t == x:
            return i
    hits = [i for i, t in enumerate(table) if t.startswith(x)]
    return hits[0] if len(hits) == 1 else None


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Dist:
    """R's ``dist`` object: the strict lower triangle of the distance
    matrix by columns, plus its attributes (Size, Labels, method, p)."""

    def __init__(self, values: np.ndarray, size: int, method: str, labels=None, p=None):
        self.values = values
        self.size = size
        self.method = method
        self.labels = labels
        self.p = p

    def __len__(self):
        return len(self.values)

    def to_matrix(self) -> np.ndarray:
        n = self.size
        m = np.zeros((n, n), dtype=self.values.dtype)
        # R's dist order is column-major over the lower triangle.
        cols, rows = np.triu_indices(n, 1)
        m[rows, cols] = self.values
        m[cols, rows] = self.values
        return m


def gpuDist(points, method: str = "euclidean", p: float = 2.0, labels=None) -> Dist:
    """Distances between the rows of ``points`` (R/gpuHclust.R:1-39)."""
    if pmatch(method, ("euclidian",)) is not None:
        method = "euclidean"
    idx = pmatch(method, DIST_METHODS)
    if idx is None:
        raise ValueError("invalid distance method")
    method = DIST_METHODS[idx]
    pts = np.asarray(points, dtype=np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(-1, 1)
    if not np.all(np.isfinite(pts)):
        # .C's default NAOK = FALSE rejects NA/NaN/Inf before the call.
        raise ValueError("NA/NaN/Inf in foreign function call (arg 1)")
    n, d = pts.shape
    rowmajor = np.ascontiguousarray(pts, dtype=np.float32)
    full = np.empty((n, n), dtype=np.float32)
    lib = load()
    if n > 0:
        check(lib.gt_distances(_ptr(rowmajor), n, d, _ptr(full), idx, float(np.float32(p))))
    # as.dist(matrix(d, N, N)): lower triangle, column by column.
    cols, rows = np.triu_indices(n, 1)
    values = full[cols, rows].astype(np.float64)
    return Dist(values, n, method, labels, p if method == "minkowski" else None)


def gpuCor(x, y=None, use: str = "everything", method: str = "pearson"):
    """Pearson or Kendall correlation of every column pair (R/gpuCor.R:1-62)."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
    size, nx = x.shape
    same = y is None
    y = x if same else np.asarray(y, dtype=np.float64)
    if y.ndim == 1:
        y = y.reshape(-1, 1)
    ny = y.shape[1]
    # pmatch(..., nomatch = -1): a miss is reported as "ambiguous", an
    # ambiguous prefix as "invalid" -- the reference's messages, verbatim.
    m = pmatch(method, COR_METHODS)
    if m is None:
        raise ValueError("ambiguous correlation method")
    u = pmatch(use, COR_USES)
    if u is None:
        raise ValueError("ambiguous correlation method")
    if y.shape[0] != size:
        raise ValueError("x and y need the same number of rows")
    # as.single(x) flattens column-major: variable j at [j*size .. j*size+size-1].
    X = np.ascontiguousarray(x.T, dtype=np.float32)
    Y = X if same else np.ascontiguousarray(y.T, dtype=np.float32)
    lib = load()
    if COR_METHODS[m] == "pearson":
        corr = np.empty((nx, ny), np.float32)
        ts = np.empty((nx, ny), np.float32)
        pairs = np.empty((nx, ny), np.float32)
        if nx and ny:
            check(lib.gt_pmcc(u, _ptr(X), nx, _ptr(Y), ny, size, _ptr(pairs), _ptr(corr), _ptr(ts)))
        return {"coefficients": corr.astype(np.float64), "ts": ts.astype(np.float64),
                "pairs": pairs.astype(np.float64)}
    if COR_USES[u] != "everything":
        warnings.warn("NA handling for Kendall's is not yet supported. Defaulting to using "
                      "everything. Sorry for any inconvenience.")
    if np.isnan(X).any() or np.isnan(Y).any():
        raise ValueError("NA/NaN/Inf in foreign function call (arg 1)")
    res = np.empty((ny, nx), np.float64)  # answers[y*nx + x]
    if nx and ny:
        check(lib.gt_kendall(_ptr(X), nx, _ptr(Y), ny, size, _ptr(res)))
    return {"coefficients": np.ascontiguousarray(res.T), "pairs": np.full((nx, ny), float(size))}


def gpuTtest(goodPairs, coeffs) -> np.ndarray:
    """t-scores of Pearson coefficients (R/gpuCor.R:64-74 via rtestT)."""
    gp = np.ascontiguousarray(np.asarray(goodPairs, dtype=np.float32).ravel())
    co = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float32).ravel())
    n = ctypes.c_int(gp.size)
    out = np.empty(gp.size, np.float32)
    lib = load()
    lib.rtestT(_ptr(gp), _ptr(co), ctypes.byref(n), _ptr(out))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return out.astype(np.float64)


def chooseGpu(deviceId: int = 0) -> int:
    """R/chooseGpu.R: select the device used by later calls."""
    lib = load()
    d = ctypes.c_int(int(deviceId))
    lib.rsetDevice(ctypes.byref(d))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return int(deviceId)


def getGpuId() -> int:
    """R/getGpuId.R: the device currently used."""
    lib = load()
    d = ctypes.c_int(-1)
    lib.rgetDevice(ctypes.byref(d))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return d.value


# ---------------------------------------------------------------------------
# Device-buffer entry points (torch tensors as the memory and stream owner).

def _stream_ptr(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def distances_device(points, method: str = "euclidean", p: float = 2.0, layout: str = "full",
                     out=None, stream=None):
    """gt_distances_device on a CUDA float32 tensor of shape (N, D)."""
    import torch
    if points.dtype != torch.float32 or not points.is_cuda or not points.is_contiguous():
        raise ValueError("points must be a contiguous float32 CUDA tensor")
    n, d = points.shape
    lay = GT_LAYOUT_FULL if layout == "full" else GT_LAYOUT_DIST
    count = n * n if lay == GT_LAYOUT_FULL else n * (n - 1) // 2
    if out is None:
        out = torch.empty(count, dtype=torch.float32, device=points.device)
    check(load().gt_distances_device(ctypes.c_void_p(points.data_ptr()), n, d,
                                     ctypes.c_void_p(out.data_ptr()), lay,
                                     DIST_METHODS.index(method), float(p), _stream_ptr(stream)))
    return out


def pmcc_device(A, B=None, use: int = 0, stream=None, outputs=("pairs", "corr", "ts")):
    """gt_pmcc_device on variable-major CUDA tensors A (nA, n) and B (nB, n);
    B None or the same tensor is the symmetric problem cor(x)."""
    import torch
    B = A if B is None else B
    nA, n = A.shape
    nB = B.shape[0]
    res = {k: torch.empty((nA, nB), dtype=torch.float32, device=A.device) for k in outputs}
    ptr = lambda k: ctypes.c_void_p(res[k].data_ptr()) if k in res else None
    check(load().gt_pmcc_device(int(use), ctypes.c_void_p(A.data_ptr()), nA,
                                ctypes.c_void_p(B.data_ptr()), nB, n, ptr("pairs"), ptr("corr"),
                                ptr("ts"), _stream_ptr(stream)))
    return res


def kendall_device(X, Y=None, stream=None):
    """gt_kendall_device on variable-major CUDA tensors; returns (ny, nx) float64."""
    import torch
    Y = X if Y is None else Y
    nx, n = X.shape
    ny = Y.shape[0]
    out = torch.empty((ny, nx), dtype=torch.float64, device=X.device)
    check(load().gt_kendall_device(ctypes.c_void_p(X.data_ptr()), nx,
                                   ctypes.c_void_p(Y.data_ptr()), ny, n,
                                   ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)))
    return out


def gpuMi(x, y=None, bins: int = 2, splineOrder: int = 1):
    """B-spline mutual information of every column pair (R/gpuMi.R): x
    (nsamples x na), y (nsamples x nb, default x).  Returns the nb x na matrix
    R builds with matrix(mi, nb, na), entry [j, i] = MI(x_i, y_j)."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
    same = y is None
    y = x if same else np.asarray(y, dtype=np.float64)
    if y.ndim == 1:
        y = y.reshape(-1, 1)
    if y.shape[0] != x.shape[0]:
        raise ValueError("x and y need the same number of samples")
    n, na = x.shape
    nb = y.shape[1]
    A = np.ascontiguousarray(x.T, dtype=np.float32)  # as.single(x): variables contiguous
    B = A if same else np.ascontiguousarray(y.T, dtype=np.float32)
    out = np.empty(na * nb, np.float32)
    check(load().gt_mutual_info(int(bins), int(splineOrder), n, A.ctypes.data_as(ctypes.c_void_p),
                                na, B.ctypes.data_as(ctypes.c_void_p), nb,
                                out.ctypes.data_as(ctypes.c_void_p)))
    return out.reshape(nb, na)


def mutual_info_device(X, Y=None, bins: int = 2, order: int = 1, stream=None):
    """gt_mutual_info_device on variable-major CUDA tensors (nx, n), (ny, n);
    returns (ny, nx) float32 with [y, x] = MI(X_x, Y_y)."""
    import torch
    Y = X if Y is None else Y
    nx, n = X.shape
    ny = Y.shape[0]
    out = torch.empty((ny, nx), dtype=torch.float32, device=X.device)
    check(load().gt_mutual_info_device(int(bins), int(order), n, ctypes.c_void_p(X.data_ptr()), nx,
                                       ctypes.c_void_p(Y.data_ptr()), ny,
                                       ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)))
    return out


class HClust:
    """R's ``hclust`` object as gpuHclust / gpuDistClust build it: merge
    ((n-1) x 2, negative = point, positive = earlier step), height, order
    (1-based leaves), labels, method, dist_method."""

    def __init__(self, merge, height, order, labels, method, dist_method):
        self.merge = merge
        self.height = height
        self.order = order
        self.labels = labels
        self.method = method
        self.dist_method = dist_method


def _hclust_method(method: str) -> str:
    idx = pmatch(method, HCLUST_METHODS)
    if idx is None:
        raise ValueError("invalid clustering method")
    return HCLUST_METHODS[idx]


def gpuHclust(distances, method: str = "complete") -> HClust:
    """Hierarchical clustering of a ``Dist`` (R/gpuHclust.R:41-90)."""
    method = _hclust_method(method)
    n = getattr(distances, "size", None)
    if n is None:
        raise ValueError("invalid dissimilarities")
    n = int(n)
    if n < 2:
        raise ValueError("must have n >= 2 objects to cluster")
    want = n * (n - 1) // 2
    if len(distances) != want:
        if len(distances) < want:
            raise ValueError("dissimilarities of improper length")
        warnings.warn("dissimilarities of improper length")
    full = np.ascontiguousarray(distances.to_matrix(), dtype=np.float32)
    if not np.all(np.isfinite(full)):
        # .C's default NAOK = FALSE rejects NA/NaN/Inf before the call
        raise ValueError("NA/NaN/Inf in foreign function call (arg 1)")
    merge = np.empty(2 * (n - 1), np.int32)
    order = np.empty(n, np.int32)
    height = np.empty(n - 1, np.float32)
    check(load().gt_hclust(_ptr(full), n, method.encode(), _ptr(merge), _ptr(order),
                           _ptr(height)))
    return HClust(merge.reshape(2, n - 1).T.copy(), height, order, distances.labels, method,
                  distances.method)


def gpuDistClust(points, distmethod: str = "euclidean", clustmethod: str = "complete",
                 labels=None) -> HClust:
    """Distances (p = 2) and clustering in one call, the distance matrix kept
    on the device (R/gpuHclust.R:92-146).  As there, "euclidian" is not an
    alias here (the reference's alias assignment names another variable)."""
    idx = pmatch(distmethod, DIST_METHODS)
    if idx is None:
        raise ValueError("invalid distance method")
    distmethod = DIST_METHODS[idx]
    clustmethod = _hclust_method(clustmethod)
    pts = np.asarray(points, dtype=np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(-1, 1)
    if not np.all(np.isfinite(pts)):
        raise ValueError("NA/NaN/Inf in foreign function call (arg 3)")
    n, d = pts.shape
    if n < 2:
        raise ValueError("must have n >= 2 objects to cluster")
    rowmajor = np.ascontiguousarray(pts, dtype=np.float32)
    merge = np.empty(2 * (n - 1), np.int32)
    order = np.empty(n, np.int32)
    height = np.empty(n - 1, np.float32)
    check(load().gt_distclust(_ptr(rowmajor), n, d, idx, clustmethod.encode(), _ptr(merge),
                              _ptr(order), _ptr(height)))
    return HClust(merge.reshape(2, n - 1).T.copy(), height, order, labels, clustmethod,
                  distmethod)


def hclust_device(D, method: str = "complete", stream=None):
    """gt_hclust_device on a contiguous float32 CUDA tensor (n, n), which is
    overwritten.  Returns numpy (merge (n-1, 2), order (n,), height (n-1,)).
    ``method`` goes to the library as is (no partial matching)."""
    import torch
    if D.dtype != torch.float32 or not D.is_cuda or not D.is_contiguous() or D.dim() != 2 \
            or D.shape[0] != D.shape[1]:
        raise ValueError("D must be a contiguous square float32 CUDA tensor")
    n = D.shape[0]
    merge = np.empty(2 * max(n - 1, 0), np.int32)
    order = np.empty(n, np.int32)
    height = np.empty(max(n - 1, 0), np.float32)
    check(load().gt_hclust_device(ctypes.c_void_p(D.data_ptr()), n, method.encode(),
                                  _ptr(merge), _ptr(order), _ptr(height), _stream_ptr(stream)))
    return merge.reshape(2, n - 1).T.copy(), order, height


def hclust_format(sub, sup):
    """gt_hclust_format: 0-based step list -> (merge (len, 2), order (len+1,))."""
    sub = np.ascontiguousarray(sub, dtype=np.int32)
    sup = np.ascontiguousarray(sup, dtype=np.int32)
    m = len(sub)
    merge = np.empty(2 * m, np.int32)
    order = np.empty(m + 1, np.int32)
    check(load().gt_hclust_format(m, _ptr(sub), _ptr(sup), _ptr(merge), _ptr(order)))
    return merge.reshape(2, m).T.copy(), order


GRAM_PATHS = {"bf16x3": _lib.GT_GRAM_TC_BF16X3, "bf16x6": _lib.GT_GRAM_TC_BF16X6,
              "fp32": _lib.GT_GRAM_FP32, "f16x3": _lib.GT_GRAM_TC_F16X3,
              "f16x6": _lib.GT_GRAM_TC_F16X6}


def set_gram_path(path: str) -> None:
    """"bf16x3" / "bf16x6" (tcgen05 split-bf16), "f16x3" (tcgen05, scaled
    split-fp16), "f16x6" (tcgen05, fixed-point fp16 digits whose products
    sum exactly: Pearson at FP64-level error) or "fp32" (CUDA cores)."""
    check(load().gt_set_gram_path(GRAM_PATHS[path]))


def get_gram_path() -> str:
    code = load().gt_get_gram_path()
    return next(k for k, v in GRAM_PATHS.items() if v == code)


# ---------------------------------------------------------------------------
# Adjoints (no counterpart in the reference): R-style gradient wrappers.

def gpuCorBackward(x, grad) -> np.ndarray:
    """dL/dx for C = cor(x) (pearson), x n x p, grad = dL/dC p x p."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
    n, p = x.shape
    X = np.ascontiguousarray(x.T, dtype=np.float32)          # as.single(x)
    G = np.ascontiguousarray(np.asarray(grad, dtype=np.float32))
    if G.shape != (p, p):
        raise ValueError("grad must be p x p")
    out = np.empty((p, n), np.float32)
    lib = load()
    lib.RgpuCorBackward(_ptr(X), ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(p)),
                        _ptr(G), _ptr(out))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return np.ascontiguousarray(out.T).astype(np.float64)


def gpuDistBackward(points, grad) -> np.ndarray:
    """dL/dpoints for the Euclidean distance matrix D, grad = dL/dD (N x N)."""
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.float32))
    n, d = pts.shape
    G = np.ascontiguousarray(np.asarray(grad, dtype=np.float32))
    if G.shape != (n, n):
        raise ValueError("grad must be N x N")
    out = np.empty((n, d), np.float32)
    lib = load()
    lib.RgpuDistBackward(_ptr(pts), ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(d)),
                         _ptr(G), _ptr(out))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return out.astype(np.float64)


def gpuMdsStress(points, delta):
    """(stress, gradient) of sum_{i<j} (D_ij - delta_ij)^2; delta a Dist or its
    values in R's dist order."""
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.float32))
    n, d = pts.shape
    dv = delta.values if isinstance(delta, Dist) else delta
    dv = np.ascontiguousarray(np.asarray(dv, dtype=np.float32))
    if dv.size != n * (n - 1) // 2:
        raise ValueError("delta must hold N(N-1)/2 values")
    out = np.empty((n, d), np.float32)
    loss = np.zeros(1, np.float64)
    lib = load()
    lib.RgpuMdsStress(_ptr(pts), ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(d)),
                      _ptr(dv), _ptr(loss), _ptr(out))
    err = _lib.last_error()
    if err:
        raise RuntimeError(err)
    return float(loss[0]), out.astype(np.float64)


# ---------------------------------------------------------------------------
# Batches (no counterpart in the reference).

class BatchPlan:
    """A batch of independent cor(x) problems (pearson or kendall) prepared
    once and replayed from a CUDA graph.  Inputs are variable-major CUDA
    float32 tensors (p, n); outputs are allocated here.  `launch()`
    recomputes every output from the current contents of the inputs.

    Pearson outputs are p x p views of pitched storage (rows a multiple of 8
    floats apart, so every row starts on a 32-byte sector) unless
    `pitched=False`, which allocates contiguous p x p tensors."""

    def __init__(self, inputs, method: str = "pearson", autotune: bool = False,
                 graph: bool = True, pitched: bool = True):
        import torch
        self.method = method
        self.inputs = list(inputs)
        lib = load()
        flags = (0 if graph else _lib.GT_BATCH_NO_GRAPH) | (_lib.GT_BATCH_AUTOTUNE if autotune else 0)
        self.outputs = []
        handle = ctypes.c_void_p()
        if method == "pearson":
            arr = (_lib.CorProblem * max(1, len(self.inputs)))()
            for i, x in enumerate(self.inputs):
                p, n = x.shape
                ld = (p + 7) // 8 * 8 if pitched else p
                o = {k: torch.empty((p, ld), dtype=torch.float32, device=x.device)[:, :p]
                     for k in ("corr", "ts", "pairs")}
                self.outputs.append(o)
                arr[i] = _lib.CorProblem(x.data_ptr(), p, n, o["corr"].data_ptr(),
                                         o["ts"].data_ptr(), o["pairs"].data_ptr(), ld)
            check(lib.gt_pmcc_batch_plan_create(arr, len(self.inputs), flags, ctypes.byref(handle)))
        elif method == "kendall":
            arr = (_lib.KendallProblem * max(1, len(self.inputs)))()
            for i, x in enumerate(self.inputs):
                p, n = x.shape
                o = torch.empty((p, p), dtype=torch.float64, device=x.device)
                self.outputs.append(o)
                arr[i] = _lib.KendallProblem(x.data_ptr(), p, n, o.data_ptr())
            check(lib.gt_kendall_batch_plan_create(arr, len(self.inputs), flags,
                                                   ctypes.byref(handle)))
        else:
            raise ValueError("method must be 'pearson' or 'kendall'")
        self._handle = handle

    def describe(self) -> str:
        d = load().gt_batch_plan_describe(self._handle)
        return d.decode() if d else ""

    def launch(self, stream=None):
        check(load().gt_batch_plan_launch(self._handle, _stream_ptr(stream)))
        return self.outputs

    def close(self):
        if self._handle:
            load().gt_batch_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
