"""gpuCor(method = "pearson") parity through the C ABI (rpmcc, gt_pmcc,
gt_pmcc_device) against the FP64 oracle.

Error metric: absolute error of r (r is already scale free, |r| <= 1).
Tolerances, per Gram evaluation:
  fp32    2e-6 * sqrt(n / 100) + 1e-6   (float32 accumulation of n products)
  bf16x6  same as fp32                  (3-way bf16 split: float32-exact products)
  bf16x3  2e-5                          (2-way split drops the lo*lo product, ~2^-16)
  f16x3   same as fp32                  (scaled 2-way fp16 split, ~2^-21 per product)
  f16x6   1.5e-7                        (fixed-point fp16 digits summed exactly: only
                                         the float rounding of r remains)
The metric's bar -- max relative error <= 1e-6 against FP64 for |r| >= 0.01 --
is asserted for f16x6 at 4096 observations (test_relative_error_bar).
pairs must match exactly; t-scores are checked against hostSignif's rule
applied to the returned r, and against the oracle away from |r| -> 1.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PATHS = ("fp32", "bf16x3", "bf16x6", "f16x3", "f16x6")


def tol(path, n):
    if path == "bf16x3":
        return 2e-5
    if path == "f16x6":
        return 1.5e-7
    return 2e-6 * np.sqrt(max(n, 1) / 100.0) + 1e-6


def rpmcc(lib, use, A, B):
    """A, B variable-major (na, n), (nb, n) -- R's as.single(x) order."""
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    na, n = A.shape
    nb = B.shape[0]
    pairs = np.full((na, nb), -1, np.float32)
    corr = np.full((na, nb), -7, np.float32)
    ts = np.full((na, nb), -7, np.float32)
    ci = lambda v: ctypes.byref(ctypes.c_int(v))
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    lib.rpmcc(ci(use), vp(A), ci(na), vp(B), ci(nb), ci(n), vp(pairs), vp(corr), vp(ts))
    err = lib.gt_last_error().decode()
    assert err == "", err
    return corr, pairs, ts


@pytest.fixture(params=PATHS)
def path(request, gpu):
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path(request.param)
    yield request.param
    g.set_gram_path(old)


def check_r(got, want, atol):
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w)
    ok = ~nan_w
    if ok.any():
        err = np.abs(got[ok].astype(np.float64) - want[ok]).max()
        assert err <= atol, err


def check_ts(ts, corr, pairs, want_ts, want_r):
    r = corr.astype(np.float32)
    rule = np.where(r >= np.float32(0.999), np.float32(10000),
                    r * np.sqrt((pairs - np.float32(2)) / (np.float32(1) - r * r)))
    ok = ~np.isnan(rule)
    np.testing.assert_allclose(ts[ok], rule[ok], rtol=2e-6, atol=1e-6)
    away = ok & (np.abs(want_r) < 0.95)
    np.testing.assert_allclose(ts[away], want_ts[away], rtol=2e-3, atol=2e-4)


@pytest.mark.parametrize("na,nb,n", [(1, 1, 3), (3, 5, 30), (37, 1, 100), (130, 70, 257),
                                     (200, 200, 64)])
def test_everything_two_sets(gpu, oracle_mod, rng, path, na, nb, n):
    A = rng.standard_normal((na, n)).astype(np.float32)
    B = (rng.standard_normal((nb, n)) * 2 + 5).astype(np.float32)
    corr, pairs, ts = rpmcc(gpu, 0, A, B)
    wc, wp, wt = oracle_mod.pearson(A, B, use=0)
    check_r(corr, wc, tol(path, n))
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_ts(ts, corr, pairs, wt, wc)


def test_fp32_large_tiles_rows_sampled(gpu, oracle_mod, rng):
    """3200 variables (one set) and 2500 x 2400 (two sets) take the 128 x 128
    tiles of the CUDA-core Gram on the FP32 path; sampled rows, the ragged
    last tile rows among them, against the oracle."""
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path("fp32")
    try:
        X = rng.standard_normal((3200, 150)).astype(np.float32)
        corr, pairs, ts = rpmcc(gpu, 0, X, X.copy())
        rows = np.concatenate([rng.choice(3072, 10, replace=False), np.arange(3190, 3200)])
        wc, wp, wt = oracle_mod.pearson(X[rows], X, use=0)
        check_r(corr[rows], wc, tol("fp32", 150))
        assert np.array_equal(corr, corr.T)
        A = rng.standard_normal((2500, 60)).astype(np.float32)
        B = (rng.standard_normal((2400, 60)) * 3 - 2).astype(np.float32)
        corr, pairs, ts = rpmcc(gpu, 0, A, B)
        rows = np.concatenate([rng.choice(2432, 10, replace=False), np.arange(2490, 2500)])
        wc, wp, wt = oracle_mod.pearson(A[rows], B, use=0)
        check_r(corr[rows], wc, tol("fp32", 60))
        assert np.array_equal(pairs, np.full_like(pairs, 60.0))
    finally:
        g.set_gram_path(old)


@pytest.mark.parametrize("p,n", [(2, 5), (65, 40), (300, 500), (513, 129)])
def test_everything_symmetric_copies(gpu, oracle_mod, rng, path, p, n):
    """gpuCor(x): R passes two copies of x through .C; the library recognises
    them and computes each unordered pair once."""
    X = rng.standard_normal((p, n)).astype(np.float32)
    corr, pairs, ts = rpmcc(gpu, 0, X, X.copy())
    wc, wp, wt = oracle_mod.pearson(X, use=0)
    check_r(corr, wc, tol(path, n))
    assert np.array_equal(corr, corr.T)
    assert np.all(np.diag(corr) == 1.0)
    assert np.all(np.diag(ts) == 10000.0)


def test_everything_nan_and_constant_columns(gpu, oracle_mod, rng, path):
    X = rng.standard_normal((50, 80)).astype(np.float32)
    X[7, 11] = np.nan
    X[9, :] = 3.25
    corr, pairs, ts = rpmcc(gpu, 0, X, X)
    wc, wp, _ = oracle_mod.pearson(X, use=0)
    check_r(corr, wc, tol(path, 80))
    assert np.all(np.isnan(corr[7])) and np.all(np.isnan(corr[:, 9]))
    assert np.all(pairs == 80)


def test_centering_stress_offsets(gpu, oracle_mod, rng, path):
    """Lognormal(5, 1) values plus per-column offsets in [0, 1e3] (the
    precision configuration's distribution, at a small size)."""
    n, p = 512, 96
    X = (rng.lognormal(5.0, 1.0, (p, n)) + rng.uniform(0, 1e3, (p, 1))).astype(np.float32)
    corr, _, _ = rpmcc(gpu, 0, X, X)
    wc, _, _ = oracle_mod.pearson(X, use=0)
    check_r(corr, wc, tol(path, n))


@pytest.mark.parametrize("na,nb,n,frac", [(4, 4, 10, 0.2), (33, 65, 200, 0.1), (120, 120, 77, 0.3)])
def test_pairwise_complete(gpu, oracle_mod, rng, na, nb, n, frac):
    A = rng.standard_normal((na, n)).astype(np.float32)
    B = rng.standard_normal((nb, n)).astype(np.float32) + 50
    A[rng.random(A.shape) < frac] = np.nan
    B[rng.random(B.shape) < frac] = np.nan
    corr, pairs, ts = rpmcc(gpu, 1, A, B)
    wc, wp, wt = oracle_mod.pearson(A, B, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_r(corr, wc, 2e-5)


@pytest.mark.parametrize("na,nb,n", [(3, 5, 30), (130, 70, 257), (200, 200, 64)])
def test_pairwise_without_missing_values(gpu, oracle_mod, rng, path, na, nb, n):
    """pairwise.complete.obs on inputs without a NaN is cor(everything): the
    tensor-core paths take it (a device NaN flag gates the launches); pairs
    are n everywhere.  A constant variable still gives NaN."""
    A = (rng.standard_normal((na, n)) * 3 + 7).astype(np.float32)
    B = (rng.standard_normal((nb, n)) + 50).astype(np.float32)
    A[1] = 4.0
    corr, pairs, ts = rpmcc(gpu, 1, A, B)
    wc, wp, wt = oracle_mod.pearson(A, B, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_r(corr, wc, tol(path, n))
    check_ts(ts, corr, pairs, wt, wc)
    # cor(x) with the same NaN-free matrix
    corr, pairs, _ = rpmcc(gpu, 1, A, A.copy())
    wc, wp, _ = oracle_mod.pearson(A, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_r(corr, wc, tol(path, n))


def test_pairwise_flag_follows_each_call(gpu, oracle_mod, rng, path):
    """Alternating inputs with and without a NaN on the same sizes: each call
    takes the right kernel (the flag is recomputed per call)."""
    A = rng.standard_normal((40, 90)).astype(np.float32)
    B = rng.standard_normal((50, 90)).astype(np.float32)
    for k in range(3):
        Bk = B.copy()
        if k == 1:
            Bk[7, 13] = np.nan
        corr, pairs, _ = rpmcc(gpu, 1, A, Bk)
        wc, wp, _ = oracle_mod.pearson(A, Bk, use=1)
        assert np.array_equal(pairs, wp.astype(np.float32))
        check_r(corr, wc, 2e-5 if k == 1 else tol(path, 90))


@pytest.mark.parametrize("frac", [0.01, 0.2])
def test_pairwise_missing_long_columns(gpu, oracle_mod, rng, path, frac):
    """Missing values over 4096 observations (16 accumulation chunks on the
    tensor cores): the same tolerance as cor(everything)."""
    n = 4096
    A = (np.exp(rng.standard_normal((150, n)) + 5.0) + rng.uniform(0, 1e3, (150, 1))).astype(np.float32)
    A[rng.random(A.shape) < frac] = np.nan
    corr, pairs, ts = rpmcc(gpu, 1, A, A.copy())
    wc, wp, wt = oracle_mod.pearson(A, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    # the masked Gram of the six sums carries the f16x3 split whatever the path
    ptol = 2e-5 if path == "bf16x3" else tol("f16x3" if path == "f16x6" else path, n)
    check_r(corr, wc, ptol)
    B = (rng.standard_normal((70, n)) - 3).astype(np.float32)
    B[rng.random(B.shape) < frac] = np.nan
    corr, pairs, _ = rpmcc(gpu, 1, A, B)
    wc, wp, _ = oracle_mod.pearson(A, B, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_r(corr, wc, ptol)


def test_pairwise_degenerate(gpu, oracle_mod):
    A = np.array([[1, np.nan, 3, 4], [np.nan, np.nan, np.nan, 2], [5, 5, 5, 5]], np.float32)
    corr, pairs, _ = rpmcc(gpu, 1, A, A.copy())
    wc, wp, _ = oracle_mod.pearson(A, use=1)
    assert np.array_equal(pairs, wp.astype(np.float32))
    check_r(corr, wc, 1e-6)


def test_status_and_device_variants_agree(gpu, rng):
    import torch
    import gputools_gb300 as g
    X = rng.standard_normal((100, 64)).astype(np.float32)
    corr, pairs, ts = rpmcc(gpu, 0, X, X)
    dX = torch.from_numpy(X).cuda()
    res = g.pmcc_device(dX)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(res["corr"].cpu().numpy(), corr)
    np.testing.assert_array_equal(res["ts"].cpu().numpy(), ts)
    np.testing.assert_array_equal(res["pairs"].cpu().numpy(), pairs)


def test_gpuCor_api(gpu, oracle_mod, rng):
    import gputools_gb300 as g
    A = rng.random((30, 5)); B = rng.random((30, 10))  # man/gpuCor.Rd example shapes
    res = g.gpuCor(A, B, method="pearson")
    wc, _, _ = oracle_mod.pearson(A.T.astype(np.float32), B.T.astype(np.float32))
    np.testing.assert_allclose(res["coefficients"], wc, atol=2e-5)
    assert res["coefficients"].shape == (5, 10) and np.all(res["pairs"] == 30)
    A[2, 1] = np.nan
    res = g.gpuCor(A, B, use="pairwise.complete.obs", method="pearson")
    assert np.all(res["pairs"][1] == 29) and np.all(res["pairs"][0] == 30)


def test_gpuTtest(gpu, rng):
    import gputools_gb300 as g
    gp = rng.poisson(5, 10) + 3
    co = rng.random(10)
    got = g.gpuTtest(gp, co)
    r = co.astype(np.float32); n = gp.astype(np.float32)
    np.testing.assert_allclose(got, r * np.sqrt((n - 2) / (1 - r * r)), rtol=2e-6)


def test_everything_large_output_pairs_from_host(gpu):
    # 8192^2 entries reach the size from which the constant pair counts of
    # "everything" are filled on the host while the device writes r and t
    nv, n = 8192, 8
    rng = np.random.default_rng(31)
    X = rng.standard_normal((nv, n)).astype(np.float32)
    pairs = np.full((nv, nv), -1.0, np.float32)
    corr = np.empty((nv, nv), np.float32)
    ts = np.empty((nv, nv), np.float32)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert gpu.gt_pmcc(0, vp(X), nv, vp(X), nv, n, vp(pairs), vp(corr), vp(ts)) == 0
    assert np.all(pairs == np.float32(n))
    rows = np.array([0, 1, 4095, 8191])
    want = np.corrcoef(X.astype(np.float64))[rows]
    assert np.max(np.abs(corr[rows] - want)) < 5e-6
    assert np.all(np.isfinite(ts[rows]))


def _rel_err(got, want, floor):
    ok = ~np.isnan(want) & (np.abs(want) >= floor)
    return float((np.abs(got[ok].astype(np.float64) - want[ok]) / np.abs(want[ok])).max())


@pytest.mark.parametrize("sym", [True, False])
def test_relative_error_bar(gpu, oracle_mod, sym):
    """Max relative error of r <= 1e-6 against the FP64 oracle for every entry
    with |r| >= 0.01, on the error-free f16x6 path, at the precision
    configuration's length and distribution (4096 observations,
    lognormal(5, 1) plus per-column offsets in [0, 1e3]), with correlated
    blocks so that |r| spans 0.01 .. 1 (near-collinear pairs included)."""
    import gputools_gb300 as g
    rng = np.random.default_rng(2024)
    n, p = 4096, 384
    base = rng.lognormal(5.0, 1.0, (p, n))
    # every 8th variable gets partners at several mixing weights
    for j in range(0, p - 7, 8):
        for t, w in enumerate((1e-4, 1e-2, 0.1, 0.5, 0.9, 3.0, 30.0)):
            base[j + 1 + t] = base[j] + w * base[j + 1 + t]
    X = (base + rng.uniform(0, 1e3, (p, 1))).astype(np.float32)
    old = g.get_gram_path()
    g.set_gram_path("f16x6")
    try:
        if sym:
            corr, _, _ = rpmcc(gpu, 0, X, X.copy())
            wc, _, _ = oracle_mod.pearson(X, use=0)
            np.fill_diagonal(wc, 1.0)
        else:
            A, B = X[: p // 2], X[p // 2 - 40:]
            corr, _, _ = rpmcc(gpu, 0, A, B)
            wc, _, _ = oracle_mod.pearson(A, B, use=0)
    finally:
        g.set_gram_path(old)
    assert np.abs(wc).max() > 0.999  # near-collinear pairs are present
    assert (np.abs(wc) < 0.02).sum() > 100  # and small correlations
    assert _rel_err(corr, wc, 0.01) <= 1e-6
    assert _rel_err(corr, wc, 0.1) <= 1e-6
    assert np.abs(corr.astype(np.float64) - wc).max() <= 1.5e-7


def test_exact_path_long_columns_and_ragged_sizes(gpu, oracle_mod, rng):
    """f16x6 over 20000 observations (exactness of the first sum does not
    depend on the length) and sizes that are not multiples of the tiles."""
    import gputools_gb300 as g
    n = 20000
    A = (rng.standard_normal((131, n)) * 1e-3 + 1e3).astype(np.float32)
    B = rng.standard_normal((257, n)).astype(np.float32)
    B[3] = A[5] * 2 - B[3] * 1e-6
    old = g.get_gram_path()
    g.set_gram_path("f16x6")
    try:
        corr, pairs, ts = rpmcc(gpu, 0, A, B)
    finally:
        g.set_gram_path(old)
    wc, wp, wt = oracle_mod.pearson(A, B, use=0)
    assert np.array_equal(pairs, wp.astype(np.float32))
    assert np.abs(corr.astype(np.float64) - wc).max() <= 1.5e-7
    assert _rel_err(corr, wc, 0.01) <= 1e-6
    check_ts(ts, corr, pairs, wt, wc)


def test_pageable_outputs_written_in_place(gpu, oracle_mod, rng):
    """Outputs from 1 MiB on in ordinary (pageable) memory, as R's .C passes
    them: written in place where the device reaches the host page tables and
    the pages are resident, else staged; either way the results match the
    oracle, and the buffers stay ordinary memory (registering them succeeds)."""
    import os
    nv, n = 1200, 96
    X = (rng.standard_normal((nv, n)) * 5 + 1).astype(np.float32)
    rows = np.array([0, 1, 599, nv - 1])
    wc, wp, _ = oracle_mod.pearson(X[rows], X)
    for k, r in enumerate(rows):
        wc[k, r] = 1.0
    cudart = ctypes.CDLL(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64",
                                      "libcudart.so"))
    for touched in (True, False):
        mk = (lambda: np.full((nv, nv), -5.0, np.float32)) if touched else \
            (lambda: np.empty((nv, nv), np.float32))
        corr, pairs, ts = mk(), mk(), mk()
        ci = lambda v: ctypes.byref(ctypes.c_int(v))
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        Xc = X.copy()
        gpu.rpmcc(ci(0), vp(X), ci(nv), vp(Xc), ci(nv), ci(n), vp(pairs), vp(corr), vp(ts))
        assert gpu.gt_last_error().decode() == ""
        assert np.abs(corr[rows].astype(np.float64) - wc).max() <= tol(gpu_path(), n)
        assert np.all(pairs == n)
        for a in (corr, pairs, ts):
            assert cudart.cudaHostRegister(a.ctypes.data_as(ctypes.c_void_p),
                                           ctypes.c_size_t(a.nbytes), 0) == 0
            assert cudart.cudaHostUnregister(a.ctypes.data_as(ctypes.c_void_p)) == 0


def gpu_path():
    import gputools_gb300 as g
    return g.get_gram_path()


@pytest.mark.parametrize("pth", ["f16x3", "f16x6"])
@pytest.mark.parametrize("sym", [True, False])
def test_banded_pipeline_into_pageable_outputs(gpu, oracle_mod, pth, sym):
    """Outputs of 64 MB and more in ordinary (pageable) memory: the Gram runs
    in bands of rows whose results host threads copy out of page-locked
    staging while the next band runs.  Checked against the oracle on rows at
    the band edges, with every pair count n and (cor(x)) an exactly
    symmetric result with a unit diagonal."""
    import gputools_gb300 as g
    rng = np.random.default_rng(4242 + sym)
    p, n = 4160, 80  # 4160 rows: 33 row blocks, so the 16 bands are uneven
    X = (rng.standard_normal((p, n)) * 3 + 100).astype(np.float32)
    X[:, :5] += np.linspace(0, 2, p, dtype=np.float32)[:, None]
    Y = X.copy() if sym else (rng.standard_normal((p, n)) + 1).astype(np.float32)
    corr = np.full((p, p), -9.0, np.float32)
    ts = np.full((p, p), -9.0, np.float32)
    pairs = np.full((p, p), -9.0, np.float32)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    old = g.get_gram_path()
    g.set_gram_path(pth)
    try:
        st = gpu.gt_pmcc(0, vp(X), p, vp(Y), p, n, vp(pairs), vp(corr), vp(ts))
    finally:
        g.set_gram_path(old)
    assert st == 0, gpu.gt_last_error().decode()
    assert np.all(pairs == n)
    rows = np.array([0, 255, 256, 511, 512, 2047, 2048, p - 129, p - 128, p - 1])
    wc, _, wt = oracle_mod.pearson(X[rows], Y, use=0)
    if sym:
        for k, r in enumerate(rows):
            wc[k, r] = 1.0
        assert np.array_equal(corr, corr.T)
        assert np.all(np.diag(corr) == 1.0)
    assert np.abs(corr[rows].astype(np.float64) - wc).max() <= tol(pth, n)
    r = corr[rows]
    rule = np.where(r >= np.float32(0.999), np.float32(10000),
                    r * np.sqrt(np.float32(n - 2) / (np.float32(1) - r * r)))
    good = ~np.isnan(rule)
    np.testing.assert_allclose(ts[rows][good], rule[good], rtol=2e-6, atol=1e-6)
