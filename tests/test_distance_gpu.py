"""gpuDist parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances are float32-level: every metric is accumulated in float32 over at
most a few hundred terms, so the relative error bound used is 2e-5
(|gpu - oracle| <= 2e-5 * max(|oracle|, 1e-3)); binary counts are exact and
only the final division rounds.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

METHODS = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")
RTOL = 2e-5


def rdistances(lib, pts, method, p=2.0):
    pts = np.ascontiguousarray(pts, np.float32)
    n, d = pts.shape
    out = np.full((n, n), np.nan, np.float32)
    N, D = ctypes.c_int(n), ctypes.c_int(d)
    m = ctypes.c_char_p(method.encode())
    pf = ctypes.c_float(p)
    lib.Rdistances(pts.ctypes.data_as(ctypes.c_void_p), ctypes.byref(N), ctypes.byref(D),
                   out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(m), ctypes.byref(pf))
    err = lib.gt_last_error().decode()
    assert err == "", err
    return out


def check_close(got, want, rtol=RTOL):
    got = np.asarray(got, np.float64)
    assert got.shape == want.shape
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w)
    inf_g, inf_w = np.isinf(got), np.isinf(want)
    assert np.array_equal(inf_g, inf_w)
    ok = ~(nan_w | inf_w)
    err = np.abs(got[ok] - want[ok]) / np.maximum(np.abs(want[ok]), 1e-3)
    assert err.size == 0 or err.max() <= rtol, float(err.max())


def data_for(method, n, d, rng):
    if method == "binary":
        return (rng.random((n, d)) < 0.3).astype(np.float32)
    return rng.standard_normal((n, d)).astype(np.float32)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("n,d", [(1, 3), (2, 1), (5, 10), (37, 13), (130, 7), (300, 64),
                                 (257, 100)])
def test_rdistances_vs_oracle(gpu, oracle_mod, rng, method, n, d):
    pts = data_for(method, n, d, rng)
    p = 3.0 if method == "minkowski" else 2.0
    got = rdistances(gpu, pts, method, p)
    want = oracle_mod.dist(pts, method, p)
    np.fill_diagonal(want, 0.0)  # the reference writes 0 on the diagonal
    check_close(got, want)
    assert np.array_equal(got, got.T)


@pytest.mark.parametrize("p", [1.0, 2.0, 3.0, 4.0, 2.5, 0.5])
def test_minkowski_powers(gpu, oracle_mod, rng, p):
    pts = rng.standard_normal((70, 9)).astype(np.float32)
    got = rdistances(gpu, pts, "minkowski", p)
    want = oracle_mod.dist(pts, "minkowski", p)
    np.fill_diagonal(want, 0.0)
    check_close(got, want, rtol=5e-5)


@pytest.mark.parametrize("p", [0.5, 2.5, 4.0, 7.0])
def test_minkowski_wide_range(gpu, oracle_mod, rng, p):
    """Coordinates over nine decades (no term leaves the float range): the
    terms 2^(p log2 |a - b|) keep the float tolerance where |p log2 |a - b||
    is large."""
    pts = (rng.standard_normal((60, 11)) * 10.0 ** rng.uniform(-5, 4, (60, 11))).astype(np.float32)
    got = rdistances(gpu, pts, "minkowski", p)
    want = oracle_mod.dist(pts, "minkowski", p)
    np.fill_diagonal(want, 0.0)
    check_close(got, want, rtol=5e-5)


def test_canberra_zero_terms_follow_R(gpu, oracle_mod, rng):
    pts = rng.standard_normal((40, 12)).astype(np.float32)
    pts[rng.random(pts.shape) < 0.4] = 0.0
    pts[3] = 0.0                       # all-zero rows: no usable term -> NaN
    pts[4] = 0.0
    pts[5, :6] = -pts[6, :6]           # a = -b != 0 -> infinite term
    got = rdistances(gpu, pts, "canberra")
    want = oracle_mod.dist(pts, "canberra")
    np.fill_diagonal(want, 0.0)
    check_close(got, want)
    assert np.isnan(got[3, 4]) and np.isinf(got[5, 6])


def test_unknown_method_string_means_euclidean(gpu, oracle_mod, rng):
    pts = rng.standard_normal((20, 4)).astype(np.float32)
    got = rdistances(gpu, pts, "dot")
    want = oracle_mod.dist(pts, "euclidean")
    check_close(got, want)


def test_duplicates_are_exactly_zero(gpu, rng):
    pts = rng.standard_normal((50, 16)).astype(np.float32)
    pts[10] = pts[20]
    for m in METHODS:
        got = rdistances(gpu, pts, m, 3.0)
        if m == "binary":
            continue
        assert got[10, 20] == 0.0 and got[20, 10] == 0.0, m


def test_cfg_4000x100_rows_sampled(gpu, oracle_mod, rng):
    """The 4000 x 100 configuration, every method, checked on sampled rows."""
    base = rng.standard_normal((4000, 100)).astype(np.float32)
    bern = (rng.random((4000, 100)) < 0.3).astype(np.float32)
    rows = rng.choice(4000, 24, replace=False)
    for m in METHODS:
        pts = bern if m == "binary" else base
        p = 3.0 if m == "minkowski" else 2.0
        got = rdistances(gpu, pts, m, p)
        want = oracle_mod.dist(pts, m, p, b=pts[rows])  # [k, x] = d(x, rows[k])
        want[np.arange(len(rows)), rows] = 0.0
        check_close(got[rows], want)


def test_large_tiles_ragged_k_rows_sampled(gpu, oracle_mod, rng):
    """3100 points take the 128 x 128 tiles of the CUDA-core engine; 17
    dimensions leave one value in the second k-slab, and 3100 = 24 x 128 + 28
    leaves a ragged last tile row."""
    base = rng.standard_normal((3100, 17)).astype(np.float32)
    base[base > 1.5] = 0.0  # zero coordinates: canberra's 0/0 terms
    bern = (rng.random((3100, 17)) < 0.3).astype(np.float32)
    rows = np.concatenate([rng.choice(3072, 12, replace=False), np.arange(3090, 3100)])
    for m in METHODS:
        pts = bern if m == "binary" else base
        p = 3.0 if m == "minkowski" else 2.0
        got = rdistances(gpu, pts, m, p)
        want = oracle_mod.dist(pts, m, p, b=pts[rows])
        want[np.arange(len(rows)), rows] = 0.0
        check_close(got[rows], want)
        assert np.array_equal(got, got.T), m


def test_device_layouts_agree(gpu, rng):
    import torch
    import gputools_gb300 as g
    pts = torch.from_numpy(rng.standard_normal((333, 24)).astype(np.float32)).cuda()
    for m in ("euclidean", "manhattan", "canberra"):
        full = g.distances_device(pts, m, layout="full").view(333, 333).cpu().numpy()
        cond = g.distances_device(pts, m, layout="dist").cpu().numpy()
        cols, rows = np.triu_indices(333, 1)
        assert np.array_equal(cond, full[cols, rows]), m
    torch.cuda.synchronize()


def test_gpuDist_api_matches_oracle(gpu, oracle_mod, rng):
    import gputools_gb300 as g
    pts = rng.random((5, 10))  # man/gpuDist.Rd example shape
    for m in ("euclidean", "maximum", "manhattan"):
        d = g.gpuDist(pts, m)
        want = oracle_mod.dist(pts.astype(np.float32), m)
        cols, rows = np.triu_indices(5, 1)
        np.testing.assert_allclose(d.values, want[cols, rows], rtol=RTOL)
        assert d.method == m and d.size == 5
    d = g.gpuDist(pts, "minkowski", 4)
    assert d.p == 4
    d = g.gpuDist(pts, "euclidian")
    assert d.method == "euclidean"


@pytest.mark.parametrize("n,d", [(200, 1000), (97, 31), (64, 32), (40, 33)])
def test_binary_exact(gpu, rng, n, d):
    # counts are exact, so the result is the float32 quotient of the two
    # integer counts, bit for bit; all-zero rows give 0, NaN counts as nonzero
    pts = (rng.random((n, d)) < 0.2).astype(np.float32)
    pts[3] = 0.0
    pts[5] = 0.0
    pts[7, ::5] = np.nan
    nz = pts != 0
    x = (nz[:, None, :] != nz[None, :, :]).sum(-1).astype(np.float32)
    o = (nz[:, None, :] | nz[None, :, :]).sum(-1).astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        want = np.where(o != 0, x / np.where(o != 0, o, 1), 0).astype(np.float32)
    np.fill_diagonal(want, 0.0)
    got = rdistances(gpu, pts, "binary")
    np.testing.assert_array_equal(got.view(np.int32), want.view(np.int32))


@pytest.mark.parametrize("n,d", [(3200, 70), (40, 70000)])
def test_binary_exact_large(gpu, rng, n, d):
    """3200 points take the 128 x 128 tiles with both counts packed in one
    accumulator; 70000 coordinates (counts past 16 bits) keep them apart.
    Bit for bit against the float32 quotient of the exact counts."""
    pts = (rng.random((n, d)) < 0.2).astype(np.float32)
    pts[3] = 0.0
    pts[7, ::5] = np.nan
    nz = (pts != 0).astype(np.float64)
    both = nz @ nz.T                       # exact: integers below 2^53
    cnt = nz.sum(1)
    x = (cnt[:, None] + cnt[None, :] - 2 * both).astype(np.float32)
    o = (cnt[:, None] + cnt[None, :] - both).astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        want = np.where(o != 0, x / np.where(o != 0, o, 1), 0).astype(np.float32)
    np.fill_diagonal(want, 0.0)
    got = rdistances(gpu, pts, "binary")
    np.testing.assert_array_equal(got.view(np.int32), want.view(np.int32))


def test_canberra_extreme_operands(gpu, oracle_mod, rng):
    # |a - b| / |a + b| at a = -b (an infinite term), with subnormal and tiny
    # magnitudes and zero coordinates: float results agree with the FP64
    # oracle to float tolerance, infinities included (sums that overflow
    # float are left out: the FP64 oracle keeps them finite)
    n, d = 48, 24
    pts = rng.standard_normal((n, d)).astype(np.float32)
    pts[1] = -pts[0]                                   # every term infinite
    pts[2, :4] = -pts[3, :4]                           # some terms infinite
    pts[4] *= np.float32(1e-39)                        # subnormal magnitudes
    pts[5] *= np.float32(3e-38)
    pts[8, ::3] = 0.0
    pts[9] = np.float32(1e-30) * pts[10]               # ratio near 1, tiny
    got = rdistances(gpu, pts, "canberra")
    want = oracle_mod.dist(pts, "canberra")
    np.fill_diagonal(want, 0.0)
    check_close(got, want)
