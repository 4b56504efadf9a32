"""The hierarchical-clustering oracle (oracle.hclust, a restatement of
src/hcluster.cpp with the kernels of inst/cuda/hcluster.cu, and
oracle.format_clustering, src/rinterface.cpp:241-290) pinned two ways:

* against scipy.cluster.hierarchy.linkage, an independent implementation of
  the same Lance-Williams schemes, where the reference's formulas are the
  textbook ones: single, complete, average, mcquitty / wpgma (scipy's
  "weighted"), and median / centroid on squared Euclidean distances (scipy
  works on their square roots);
* against a second, pure-Python reading of the reference for small cases
  (every method, ties included), bit for bit: numpy float32 / float64 scalars
  round every operation on its own, as the oracle's C (built with
  -ffp-contract=off) does.

The reference's ward update weights d(kept, k) by (|merged-away| + |k|)
(inst/cuda/hcluster.cu:388), the transpose of the textbook weights, so ward
is pinned by the Python reading only.  The gt_hclust_format tests check the
library's O(n) host formatter against the oracle's O(n^2) one (no GPU).
"""
import math

import numpy as np
import pytest

import oracle

METHODS = ["single", "complete", "average", "mcquitty", "wpgma", "median", "centroid",
           "flexible", "flexible_group", "ward"]

f32, f64 = np.float32, np.float64


def _before(v1, c1, v2, c2):
    if v1 < v2:
        return True
    if not v1 == v2:
        return False
    if (c1 & 31) != (c2 & 31):
        return (c1 & 31) < (c2 & 31)
    return c1 < c2


def _update(m, top, bot, nr, np_, nk, val):
    """inst/cuda/hcluster.cu:108-401, one column, lambda = beta = 0.5."""
    with np.errstate(all="ignore"):  # inf * 0 in ward on retired columns
        return _update_raw(m, top, bot, nr, np_, nk, val)


def _update_raw(m, top, bot, nr, np_, nk, val):
    nq = f32(nr - np_)
    lam, beta = f32(0.5), f32(0.5)
    if m == "single":
        return min(bot, top)
    if m == "complete":
        return max(bot, top)
    if m in ("mcquitty", "wpgma"):
        return f32(f64(f32(bot + top)) / 2.0)
    if m == "average":
        return f32(f32(f32(top * np_) + f32(bot * nq)) / nr)
    if m == "median":
        return f32(f64(f64(f32(bot + top)) / 2.0) - f64(f64(val) / 4.0))
    if m == "centroid":
        t1 = f32(f32(f32(top * np_) + f32(bot * nq)) / nr)
        t2 = f32(f32(f32(np_ * nq) * val) / f32(nr * nr))
        return f32(t1 - t2)
    if m == "flexible_group":
        l1 = f64(1.0 - f64(lam))
        a = f64(f64(f64(bot) * l1) * f64(np_))
        b = f64(f64(f64(top) * l1) * f64(nq))
        return f32(f64(f64(a + b) / f64(nr)) + f64(f32(beta * val)))
    if m == "flexible":
        l1 = f64(1.0 - f64(lam))
        a, b = f64(f64(bot) * l1), f64(f64(top) * l1)
        return f32(f64(f64(a + b) / 2.0) + f64(f32(beta * val)))
    if m == "ward":
        a = f32(bot * f32(np_ + nk))
        b = f32(top * f32(nq + nk))
        v = f32(f32(f32(a + b) - f32(val * nk)) / f32(nr + nk))
        return f32(math.inf) if math.isinf(v) else v
    raise ValueError(m)


def python_hclust(D, m):
    """The reference's loop (src/hcluster.cpp:40-201) for small n."""
    n = D.shape[0]
    d = [[f32(D[i, j]) for j in range(n)] for i in range(n)]
    inf = f32(math.inf)
    for i in range(n):
        d[i][i] = inf
    cnt = [f32(1.0)] * n
    sub, sup, val = [], [], []
    for _ in range(n - 1):
        mv, mc = [inf] * n, [0] * n
        for row in range(n):
            if cnt[row] > 0:
                for col in range(row + 1):
                    if _before(d[row][col], col, mv[row], mc[row]):
                        mv[row], mc[row] = d[row][col], col
        bv, br = inf, 0
        for row in range(n):
            if cnt[row] > 0 and _before(mv[row], row, bv, br):
                bv, br = mv[row], row
        c, r = mc[br], br
        sub.append(c), sup.append(r), val.append(bv)
        cnt[r] = f32(cnt[r] + cnt[c])
        cnt[c] = f32(-cnt[c])
        nr, np_ = cnt[r], f32(-cnt[c])
        new = []
        for col in range(n):
            if col == c or col == r or (m == "ward" and nr == -cnt[col]):
                new.append(inf)
            else:
                new.append(_update(m, d[c][col], d[r][col], nr, np_, cnt[col], bv))
        for col in range(n):
            d[r][col] = d[col][r] = new[col]
        for col in range(n):
            d[c][col] = d[col][c] = inf
    return np.array(sub), np.array(sup), np.array(val, np.float32)


def sym(rng, n, ties=False, sq_euclid=False):
    if sq_euclid:
        x = rng.standard_normal((n, 3))
        D = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    else:
        D = rng.random((n, n))
        D = (D + D.T) / 2
    if ties:
        D = np.round(D * 3)
    D = D.astype(np.float32)
    np.fill_diagonal(D, 0)
    return D


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("ties", [False, True])
def test_oracle_matches_python_reading(method, ties):
    rng = np.random.default_rng(7 + METHODS.index(method) + 100 * ties)
    for n in (2, 3, 9, 37):
        D = sym(rng, n, ties=ties)
        s1, p1, v1 = oracle.hclust(D, method)
        s2, p2, v2 = python_hclust(D, method)
        np.testing.assert_array_equal(s1, s2)
        np.testing.assert_array_equal(p1, p2)
        np.testing.assert_array_equal(v1.view(np.int32), v2.view(np.int32))


def test_unknown_names_are_single_linkage():
    rng = np.random.default_rng(3)
    D = sym(rng, 20)
    ref = oracle.hclust(D, "single")
    for name in ("flexible group", "nonsense", ""):
        got = oracle.hclust(D, name)
        for a, b in zip(ref, got):
            np.testing.assert_array_equal(a, b)


hier = pytest.importorskip("scipy.cluster.hierarchy")
dist = pytest.importorskip("scipy.spatial.distance")


def _scipy(D, method):
    return hier.linkage(dist.squareform(D.astype(np.float64), checks=False), method=method)


@pytest.mark.parametrize("method,scipy_method", [("single", "single"), ("complete", "complete"),
                                                 ("average", "average"),
                                                 ("mcquitty", "weighted"), ("wpgma", "weighted")])
def test_oracle_heights_match_scipy(method, scipy_method):
    rng = np.random.default_rng(11)
    for n in (5, 40, 120):
        D = sym(rng, n)
        _, _, val = oracle.hclust(D, method)
        Z = _scipy(D, scipy_method)
        np.testing.assert_allclose(np.sort(val), np.sort(Z[:, 2]), rtol=2e-6, atol=1e-7)


@pytest.mark.parametrize("method", ["median", "centroid"])
def test_oracle_squared_euclid_schemes_match_scipy(method):
    rng = np.random.default_rng(12)
    for n in (6, 30, 80):
        D = sym(rng, n, sq_euclid=True)
        _, _, val = oracle.hclust(D, method)
        Z = _scipy(np.sqrt(D.astype(np.float64)), method)
        np.testing.assert_allclose(val, Z[:, 2] ** 2, rtol=1e-4, atol=1e-5)


def test_oracle_merge_sets_match_scipy():
    # the same clusters form, whatever the order of equal-height merges
    rng = np.random.default_rng(13)
    D = sym(rng, 60)
    sub, sup, _ = oracle.hclust(D, "average")
    merge, order = oracle.format_clustering(sub, sup)
    Z = _scipy(D, "average")

    def clusters(pairs, n):
        members = {}
        out = set()
        for j, (a, b) in enumerate(pairs):
            s = set()
            for v in (a, b):
                s |= members[v] if v in members else {v}
            members[n + j] = s
            out.add(frozenset(s))
        return out

    n = D.shape[0]
    ours = [(int(-a - 1) if a < 0 else n + a - 1, int(-b - 1) if b < 0 else n + b - 1)
            for a, b in merge]
    theirs = [(int(a), int(b)) for a, b in Z[:, :2]]
    assert clusters(ours, n) == clusters(theirs, n)
    assert sorted(order.tolist()) == list(range(1, n + 1))


# ---- the library's host formatter (no GPU involved) ------------------------

@pytest.fixture(scope="module")
def gt():
    import gputools_gb300 as g
    g.load()
    return g


@pytest.mark.parametrize("method", METHODS)
def test_host_format_matches_oracle(gt, method):
    rng = np.random.default_rng(21 + METHODS.index(method))
    for n in (2, 3, 17, 150):
        D = sym(rng, n, ties=(n == 17))
        sub, sup, _ = oracle.hclust(D, method)
        m1, o1 = oracle.format_clustering(sub, sup)
        m2, o2 = gt.hclust_format(sub, sup)
        np.testing.assert_array_equal(m1, m2)
        np.testing.assert_array_equal(o1, o2)


def test_host_format_rejects_non_trees(gt):
    with pytest.raises(Exception):
        gt.hclust_format([0, 0], [1, 1])  # the same pair twice
    with pytest.raises(Exception):
        gt.hclust_format([0], [5])  # index outside 0..len


def test_gpuHclust_argument_checks(gt):
    # R/gpuHclust.R's checks, raised before the library is called
    from gputools_gb300.api import Dist
    d = Dist(np.array([1.0, 2.0, 3.0]), 3, "euclidean")
    with pytest.raises(ValueError, match="invalid clustering method"):
        gt.gpuHclust(d, "nonsense")
    with pytest.raises(ValueError, match="invalid clustering method"):
        gt.gpuHclust(d, "flex")  # ambiguous between flexible and flexible group
    with pytest.raises(ValueError, match="n >= 2"):
        gt.gpuHclust(Dist(np.array([]), 1, "euclidean"))
    with pytest.raises(ValueError, match="improper length"):
        gt.gpuHclust(Dist(np.array([1.0, 2.0]), 3, "euclidean"))
    with pytest.raises(ValueError, match="NA/NaN/Inf"):
        gt.gpuHclust(Dist(np.array([1.0, np.inf, 3.0]), 3, "euclidean"))
    with pytest.raises(ValueError, match="invalid distance method"):
        gt.gpuDistClust(np.zeros((3, 2)), "euclidian")  # the alias does not reach distmethod
    with pytest.raises(ValueError, match="NA/NaN/Inf"):
        gt.gpuDistClust(np.array([[0.0, np.nan], [1.0, 2.0]]))
