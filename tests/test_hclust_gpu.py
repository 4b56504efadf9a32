"""gpuHclust / gpuDistClust through the C ABI against the oracle
(oracle.hclust + oracle.format_clustering, pinned in test_oracle_hclust.py).

The device loop evaluates the same Lance-Williams expressions with every
operation rounded on its own and breaks ties by the same key, so merges,
leaf order and heights must be identical: heights are compared bit for bit.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

METHODS = ["single", "complete", "average", "mcquitty", "wpgma", "median", "centroid",
           "flexible", "flexible_group", "ward"]


def sym(rng, n, kind="uniform"):
    if kind == "points":
        x = rng.standard_normal((n, 4))
        D = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    else:
        D = rng.random((n, n))
        D = (D + D.T) / 2
        if kind == "ties":
            D = np.round(D * 4)
    D = D.astype(np.float32)
    np.fill_diagonal(D, 0)
    return D


def want(oracle_mod, D, method):
    sub, sup, val = oracle_mod.hclust(D, method)
    merge, order = oracle_mod.format_clustering(sub, sup)
    return merge, order, val


def same(got, ref):
    merge, order, height = got
    m2, o2, h2 = ref
    np.testing.assert_array_equal(merge, m2)
    np.testing.assert_array_equal(order, o2)
    np.testing.assert_array_equal(np.asarray(height, np.float32).view(np.int32),
                                  np.asarray(h2, np.float32).view(np.int32))


def run_host(lib, D, method):
    n = D.shape[0]
    merge = np.empty(2 * (n - 1), np.int32)
    order = np.empty(n, np.int32)
    height = np.empty(n - 1, np.float32)
    D = np.ascontiguousarray(D, np.float32)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = lib.gt_hclust(vp(D), n, method.encode(), vp(merge), vp(order), vp(height))
    assert rc == 0
    return merge.reshape(2, n - 1).T, order, height


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("kind", ["uniform", "ties", "points"])
def test_hclust_matches_oracle(gpu, oracle_mod, method, kind):
    rng = np.random.default_rng(100 + METHODS.index(method))
    for n in (2, 3, 33, 300):
        D = sym(rng, n, kind)
        same(run_host(gpu, D, method), want(oracle_mod, D, method))


@pytest.mark.parametrize("method", ["single", "average", "ward", "centroid"])
def test_hclust_ragged_size(gpu, oracle_mod, method):
    # 1500 points: not a multiple of 32 nor of the 16 CTAs' slices
    rng = np.random.default_rng(7)
    D = sym(rng, 1500, "points")
    same(run_host(gpu, D, method), want(oracle_mod, D, method))


def test_hclust_infinite_distances(gpu, oracle_mod):
    # two groups at infinite distance: the last merge is at +inf, and the
    # degenerate all-infinite rows must still follow the reference's keys
    rng = np.random.default_rng(8)
    D = sym(rng, 40)
    D[:20, 20:] = np.inf
    D[20:, :20] = np.inf
    for method in METHODS:
        same(run_host(gpu, D, method), want(oracle_mod, D, method))


def test_unknown_method_names_are_single(gpu, oracle_mod):
    rng = np.random.default_rng(9)
    D = sym(rng, 50)
    ref = want(oracle_mod, D, "single")
    for name in ("flexible group", "Ward", "xyz"):
        same(run_host(gpu, D, name), ref)


def test_gpuHclust_api(gpu, oracle_mod):
    import gputools_gb300 as g
    rng = np.random.default_rng(10)
    pts = rng.standard_normal((64, 5)).astype(np.float32)
    d = g.gpuDist(pts)
    full = d.to_matrix().astype(np.float32)
    for method in ("complete", "ave", "flexible group", "ward"):
        res = g.gpuHclust(d, method)
        m = g.api.HCLUST_METHODS[g.pmatch(method, g.api.HCLUST_METHODS)]
        same((res.merge, res.order, res.height), want(oracle_mod, full, m))
        assert res.dist_method == "euclidean"
    with pytest.raises(ValueError):
        g.gpuHclust(d, "flex")  # ambiguous prefix
    with pytest.raises(ValueError):
        g.gpuHclust(g.gpuDist(pts[:1]))


def test_Rhcluster_entry_point(gpu, oracle_mod):
    rng = np.random.default_rng(11)
    n = 45
    D = sym(rng, n)
    merge = np.empty(2 * (n - 1), np.int32)
    order = np.empty(n, np.int32)
    val = np.empty(n - 1, np.float32)
    meth = (ctypes.c_char_p * 1)(b"average")
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    gpu.Rhcluster(vp(D), ctypes.byref(ctypes.c_int(n)), vp(merge), vp(order), vp(val), meth)
    same((merge.reshape(2, n - 1).T, order, val), want(oracle_mod, D, "average"))


def test_hclust_device(gpu, oracle_mod):
    import torch

    import gputools_gb300 as g
    rng = np.random.default_rng(12)
    D = sym(rng, 700, "points")
    t = torch.from_numpy(D).cuda()
    same(g.hclust_device(t, "complete"), want(oracle_mod, D, "complete"))


@pytest.mark.parametrize("distmethod", ["euclidean", "manhattan", "maximum"])
def test_gpuDistClust_matches_oracle_on_its_distances(gpu, oracle_mod, distmethod):
    import torch

    import gputools_gb300 as g
    rng = np.random.default_rng(13)
    pts = rng.standard_normal((257, 16)).astype(np.float32)
    full = g.distances_device(torch.from_numpy(pts).cuda(), distmethod).cpu().numpy()
    full = full.reshape(257, 257)
    for method in ("complete", "average", "median"):
        res = g.gpuDistClust(pts, distmethod, method)
        same((res.merge, res.order, res.height), want(oracle_mod, full, method))


def test_Rdistclust_entry_point(gpu, oracle_mod):
    import gputools_gb300 as g
    rng = np.random.default_rng(14)
    n, dim = 80, 7
    pts = rng.random((n, dim)).astype(np.float32)
    merge = np.empty(2 * (n - 1), np.int32)
    order = np.empty(n, np.int32)
    val = np.empty(n - 1, np.float32)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    gpu.Rdistclust((ctypes.c_char_p * 1)(b"canberra"), (ctypes.c_char_p * 1)(b"single"), vp(pts),
                   ctypes.byref(ctypes.c_int(n)), ctypes.byref(ctypes.c_int(dim)), vp(merge),
                   vp(order), vp(val))
    full = np.empty((n, n), np.float32)
    assert gpu.gt_distances(vp(pts), n, dim, vp(full), 3, 2.0) == 0
    same((merge.reshape(2, n - 1).T, order, val), want(oracle_mod, full, "single"))


def test_gpuDistClust_well_separated_clusters(gpu):
    import gputools_gb300 as g
    rng = np.random.default_rng(15)
    centers = rng.standard_normal((5, 8)) * 50
    pts = (centers[np.repeat(np.arange(5), 40)] + rng.standard_normal((200, 8))).astype(np.float32)
    res = g.gpuDistClust(pts, "euclidean", "average")
    # the last four merges join the five blobs
    assert np.all(np.diff(res.height) >= -1e-6)
    assert res.height[-5] < 10 < res.height[-4]
    assert sorted(res.order.tolist()) == list(range(1, 201))


@pytest.mark.parametrize("ctas", ["1", "3", "7", "16"])
@pytest.mark.parametrize("counts", ["auto", "owned"])
def test_hclust_cluster_sizes_and_count_layouts(gpu, oracle_mod, monkeypatch, ctas, counts):
    # the merges do not depend on how the indices are split over the CTAs, nor
    # on where the counts live (all of them in every CTA, or each CTA its own
    # and the others read through distributed shared memory -- the layout
    # used above ~40000 points)
    monkeypatch.setenv("GT_HCLUST_CTAS", ctas)
    if counts == "owned":
        monkeypatch.setenv("GT_HCLUST_COUNTS", "owned")
    rng = np.random.default_rng(16)
    for n, kind in ((1100, "points"), (257, "ties")):
        D = sym(rng, n, kind)
        for method in ("average", "ward", "single"):
            same(run_host(gpu, D, method), want(oracle_mod, D, method))
    D = sym(rng, 90)
    D[:45, 45:] = np.inf
    D[45:, :45] = np.inf
    same(run_host(gpu, D, "centroid"), want(oracle_mod, D, "centroid"))


@pytest.mark.parametrize("method", ["single", "complete"])
def test_hclust_asymmetric_matrix(gpu, oracle_mod, method):
    # the C ABI takes any n x n matrix: an asymmetric one is clustered as the
    # reference would (row c and the lower triangle are read), and single
    # linkage's shortcut for symmetric matrices stays off
    rng = np.random.default_rng(17)
    for n in (40, 700):
        D = rng.random((n, n)).astype(np.float32)
        np.fill_diagonal(D, 0)
        same(run_host(gpu, D, method), want(oracle_mod, D, method))
    D = sym(rng, 300, "ties")
    D[5, 7] += 0.5  # one entry off
    same(run_host(gpu, D, "single"), want(oracle_mod, D, "single"))
