"""The FP64 oracle adjoints against FP64 central finite differences on the
64 x 32 sub-problem (CPU only).  The GPU adjoint kernels are then checked
against these oracles in tests/test_backward_gpu.py."""
import numpy as np
import pytest
from scipy.spatial.distance import cdist

H = 1e-6


def fd_grad(f, X):
    g = np.zeros_like(X)
    it = np.nditer(X, flags=["multi_index"])
    for _ in it:
        i = it.multi_index
        x0 = X[i]
        X[i] = x0 + H
        fp = f(X)
        X[i] = x0 - H
        fm = f(X)
        X[i] = x0
        g[i] = (fp - fm) / (2 * H)
    return g


def test_cor_backward_vs_finite_differences(oracle_mod):
    rng = np.random.default_rng(1)
    p, n = 32, 64                               # 64 observations x 32 variables
    X32 = rng.standard_normal((p, n)).astype(np.float32)
    G = rng.standard_normal((p, p))
    G = G + G.T                                 # symmetric upstream, as dL/dC of a loss on cor(x)
    X = X32.astype(np.float64)
    loss = lambda Y: float(np.sum(G * np.corrcoef(Y)))
    want = fd_grad(loss, X.copy())
    got = oracle_mod.cor_backward(X32, G)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_cor_backward_nonsymmetric_upstream(oracle_mod):
    rng = np.random.default_rng(2)
    p, n = 9, 30
    X32 = (rng.standard_normal((p, n)) * 3 + 40).astype(np.float32)
    G = rng.standard_normal((p, p))
    X = X32.astype(np.float64)
    loss = lambda Y: float(np.sum(G * np.corrcoef(Y)))
    want = fd_grad(loss, X.copy())
    got = oracle_mod.cor_backward(X32, G)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_dist_backward_vs_finite_differences(oracle_mod):
    rng = np.random.default_rng(3)
    n, d = 64, 32
    X32 = rng.standard_normal((n, d)).astype(np.float32)
    G = rng.standard_normal((n, n))
    X = X32.astype(np.float64)
    loss = lambda Y: float(np.sum(G * cdist(Y, Y)))
    want = fd_grad(loss, X.copy())
    got = oracle_mod.dist_backward(X32, G)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_mds_stress_vs_finite_differences(oracle_mod):
    rng = np.random.default_rng(4)
    n, d = 64, 32
    X32 = rng.standard_normal((n, d)).astype(np.float32)
    T = rng.standard_normal((n, d))
    cols, rows = np.triu_indices(n, 1)
    delta = cdist(T, T)[cols, rows].astype(np.float32)   # R dist order
    X = X32.astype(np.float64)

    def loss(Y):
        D = cdist(Y, Y)[cols, rows]
        return float(np.sum((D - delta.astype(np.float64)) ** 2))

    want = fd_grad(loss, X.copy())
    L, got = oracle_mod.mds_stress(X32, delta)
    assert L == pytest.approx(loss(X), rel=1e-12)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
