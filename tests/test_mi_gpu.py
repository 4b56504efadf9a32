"""gpuMi (B-spline mutual information) through the C ABI against the FP64
oracle (pinned to an independent B-spline implementation in
test_oracle_mi.py).

Up to 32 bins the joint probabilities come from an f16x3 tensor-core Gram of
the weights (~2^-21 per product) and the epilogue sums p log2 p with the
hardware log2; more bins, and the FP32 path, use CUDA cores.  Tolerance:
|got - want| <= 3e-5 + 1e-4 |want| (MI and entropies are O(1) bits).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def close(got, want):
    err = np.abs(got.astype(np.float64) - want)
    assert np.all(err <= 3e-5 + 1e-4 * np.abs(want)), float(err.max())


def data(rng, nv, n, kind="normal"):
    if kind == "normal":
        return rng.standard_normal((nv, n)).astype(np.float32)
    if kind == "skew":
        return np.exp(rng.standard_normal((nv, n)) * 1.5).astype(np.float32)
    base = rng.standard_normal((1, n))
    return (base + 0.3 * rng.standard_normal((nv, n))).astype(np.float32)  # dependent


@pytest.mark.parametrize("bins,order", [(1, 1), (2, 1), (3, 2), (10, 3), (16, 4), (32, 3), (7, 7)])
@pytest.mark.parametrize("n", [1, 37, 1000])
def test_symmetric(gpu, oracle_mod, rng, bins, order, n):
    import gputools_gb300 as g
    X = data(rng, 50, n, "dependent")
    want, _, _ = oracle_mod.bspline_mi(X, bins=bins, order=order)
    got = g.gpuMi(X.T, bins=bins, splineOrder=order)
    close(got, want)


@pytest.mark.parametrize("bins,order", [(2, 1), (10, 3), (13, 2)])
def test_two_sets(gpu, oracle_mod, rng, bins, order):
    import gputools_gb300 as g
    X = data(rng, 70, 513, "skew")
    Y = data(rng, 45, 513, "normal")
    want, _, _ = oracle_mod.bspline_mi(X, Y, bins=bins, order=order)
    got = g.gpuMi(X.T, Y.T, bins=bins, splineOrder=order)
    assert got.shape == (45, 70)
    close(got, want)


def test_many_variables_and_samples(gpu, oracle_mod, rng):
    """Several tiles of the Gram (600 variables x 16 bins = 9600 rows) and
    K chunks (4097 samples)."""
    import gputools_gb300 as g
    X = data(rng, 600, 4097, "dependent")
    got = g.gpuMi(X.T, bins=16, splineOrder=3)
    rows = np.array([0, 1, 77, 300, 599])
    want, _, _ = oracle_mod.bspline_mi(X, X[rows], bins=16, order=3)
    close(got[rows], want)


@pytest.mark.parametrize("bins", [33, 40])
def test_cuda_core_path_many_bins(gpu, oracle_mod, rng, bins):
    import gputools_gb300 as g
    X = data(rng, 20, 300, "dependent")
    want, _, _ = oracle_mod.bspline_mi(X, bins=bins, order=3)
    close(g.gpuMi(X.T, bins=bins, splineOrder=3), want)


def test_fp32_path(gpu, oracle_mod, rng):
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path("fp32")
    try:
        X = data(rng, 30, 200, "dependent")
        want, _, _ = oracle_mod.bspline_mi(X, bins=10, order=3)
        close(g.gpuMi(X.T, bins=10, splineOrder=3), want)
    finally:
        g.set_gram_path(old)


def test_constant_variable(gpu, oracle_mod, rng):
    """max == min: scaled to zeros (all weight in the first bins)."""
    import gputools_gb300 as g
    X = data(rng, 6, 120)
    X[2] = 3.5
    want, _, _ = oracle_mod.bspline_mi(X, bins=5, order=2)
    close(g.gpuMi(X.T, bins=5, splineOrder=2), want)


def test_dotC_entry_and_device(gpu, oracle_mod, rng):
    import torch
    import gputools_gb300 as g
    lib = gpu
    X = data(rng, 40, 250, "dependent")
    Y = data(rng, 40, 250, "skew")
    want, _, _ = oracle_mod.bspline_mi(X, Y, bins=8, order=2)
    out = np.full(40 * 40, -1, np.float32)
    ci = lambda v: ctypes.byref(ctypes.c_int(v))
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    lib.rBSplineMutualInfo(ci(8), ci(2), ci(250), ci(40), vp(X), ci(40), vp(Y), vp(out))
    assert lib.gt_last_error().decode() == ""
    close(out.reshape(40, 40), want)  # [y * rowsA + x]
    d = g.mutual_info_device(torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda(), bins=8, order=2)
    torch.cuda.synchronize()
    close(d.cpu().numpy(), want)


@pytest.mark.parametrize("bins,order", [(0, 1), (3, 0), (3, 4), (20, 9)])
def test_bad_arguments(gpu, rng, bins, order):
    import gputools_gb300 as g
    X = data(rng, 3, 10)
    with pytest.raises(g.GpuToolsError):
        g.gpuMi(X.T, bins=bins, splineOrder=order)
