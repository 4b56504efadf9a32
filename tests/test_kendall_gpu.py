"""gpuCor(method = "kendall") parity: bit-exact against the oracle's tau-b.

Kendall's counts are integers, so the GPU result must equal the oracle's
double S / (sqrt(Tx) * sqrt(Ty)) exactly (NaN where a variable is constant).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rgpukendall(lib, X, Y):
    X = np.ascontiguousarray(X, np.float32); Y = np.ascontiguousarray(Y, np.float32)
    nx, n = X.shape
    ny = Y.shape[0]
    out = np.full((ny, nx), -5.0)
    ci = lambda v: ctypes.byref(ctypes.c_int(v))
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    lib.RgpuKendall(vp(X), ci(nx), vp(Y), ci(ny), ci(n), vp(out))
    err = lib.gt_last_error().decode()
    assert err == "", err
    return out


def same_bits(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(
        a[~np.isnan(a)], b[~np.isnan(b)])


@pytest.mark.parametrize("n", [2, 3, 4, 5, 31, 32, 33, 64, 65, 200, 500])
def test_heavy_ties_two_sets_bit_exact(gpu, oracle_mod, rng, n):
    X = rng.integers(0, 10, (13, n)).astype(np.float32)
    Y = rng.integers(0, 4, (7, n)).astype(np.float32)
    got = rgpukendall(gpu, X, Y)
    want, *_ = oracle_mod.kendall(X, Y)
    assert same_bits(got, want)


@pytest.mark.parametrize("p,n", [(1, 10), (70, 101), (130, 64), (200, 500)])
def test_symmetric_copies_bit_exact(gpu, oracle_mod, rng, p, n):
    X = rng.integers(0, 10, (p, n)).astype(np.float32)
    got = rgpukendall(gpu, X, X.copy())
    want, *_ = oracle_mod.kendall(X)
    assert same_bits(got, want)
    assert np.all(np.diag(got) == 1.0)


def test_continuous_and_constant(gpu, oracle_mod, rng):
    X = rng.standard_normal((20, 77)).astype(np.float32)
    X[5] = 2.0
    Y = rng.standard_normal((9, 77)).astype(np.float32)
    got = rgpukendall(gpu, X, Y)
    want, *_ = oracle_mod.kendall(X, Y)
    assert same_bits(got, want)
    assert np.all(np.isnan(got[:, 5]))


def test_reference_example_shape_and_device_variant(gpu, oracle_mod, rng):
    import torch
    import gputools_gb300 as g
    A = rng.random((30, 5)); B = rng.random((30, 10))  # man/gpuCor.Rd example
    res = g.gpuCor(A, B, method="kendall")
    want, *_ = oracle_mod.kendall(A.T.astype(np.float32), B.T.astype(np.float32))
    assert same_bits(res["coefficients"], want.T)
    assert np.all(res["pairs"] == 30)
    dX = torch.from_numpy(np.ascontiguousarray(A.T, dtype=np.float32)).cuda()
    out = g.kendall_device(dX).cpu().numpy()
    w2, *_ = oracle_mod.kendall(A.T.astype(np.float32))
    assert same_bits(out, w2)


def test_cfg_500x1000_sampled(gpu, oracle_mod, rng):
    """The 500-observation, 1000-variable heavy-tie configuration, checked
    bit-exactly on a sampled block of variable pairs."""
    X = rng.integers(0, 10, (1000, 500)).astype(np.float32)
    got = rgpukendall(gpu, X, X.copy())
    cols = rng.choice(1000, 12, replace=False)
    rows = rng.choice(1000, 9, replace=False)
    want, *_ = oracle_mod.kendall(X[cols], X[rows], same=False)  # [k, j] = tau(X[cols[j]], X[rows[k]])
    sub = got[np.ix_(rows, cols)]
    for k in range(len(rows)):
        for j in range(len(cols)):
            if rows[k] == cols[j]:
                want[k, j] = 1.0
    assert same_bits(sub, want)
