"""The B-spline mutual-information oracle (oracle.bspline_mi, a restatement
of src/mi.cpp + inst/cuda/mi.cu) pinned against an independent
implementation: scipy's B-spline design matrix on the same clamped knot
vector (order zeros, 1 .. nbins - order, then nbins - order + 1 repeated),
the samples scaled to [0, nbins - order + 1] in float32 as the reference's
scale() does, and entropies / MI in numpy FP64; order 1 is also checked
against a plain joint histogram.
"""
import numpy as np
import pytest

scipy_interp = pytest.importorskip("scipy.interpolate")


def knots(nbins, order):
    t = np.zeros(nbins + order)
    for i in range(nbins + order):
        if i <= order - 1:
            t[i] = 0.0
        elif i <= nbins - 1:
            t[i] = t[i - 1] + 1.0
        else:
            t[i] = t[nbins - 1] + 1.0
    return t


def scaled(x, nbins, order):
    x = x.astype(np.float32)
    mn, mx = x.min(), x.max()
    kmax = np.float32(nbins - order + 1)
    return (kmax * (x - mn)) / (mx - mn)


def weights(x, nbins, order):
    z = scaled(x, nbins, order).astype(np.float64)
    t = knots(nbins, order)
    if order == 1:
        idx = np.minimum(np.floor(z).astype(int), nbins - 1)
        w = np.zeros((z.size, nbins))
        w[np.arange(z.size), idx] = 1.0
        return w
    # every basis function at z; the float32 scaling can put the maximum a
    # rounding above the last knot, where the reference's last interval
    # polynomial (extrapolated) applies
    return scipy_interp.BSpline(t, np.eye(nbins), order - 1, extrapolate=True)(z)


def mi_independent(X, Y, nbins, order):
    n = X.shape[1]
    wx = [weights(x, nbins, order) for x in X]
    wy = [weights(y, nbins, order) for y in Y]
    ent = lambda p: -np.sum(np.where(p > 0, p * np.log2(np.where(p > 0, p, 1)), 0.0))
    hx = np.array([ent(w.sum(0) / n) for w in wx])
    hy = np.array([ent(w.sum(0) / n) for w in wy])
    out = np.empty((len(Y), len(X)))
    for j, b in enumerate(wy):
        for i, a in enumerate(wx):
            p = a.T @ b / n
            out[j, i] = -ent(p) + hx[i] + hy[j]
    return out, hx, hy


@pytest.mark.parametrize("nbins,order", [(2, 1), (5, 1), (10, 3), (7, 2), (16, 4), (3, 3)])
def test_oracle_matches_independent_bsplines(oracle_mod, nbins, order):
    rng = np.random.default_rng(nbins * 10 + order)
    X = rng.standard_normal((6, 157)).astype(np.float32)
    Y = (rng.standard_normal((4, 157)) ** 3).astype(np.float32)
    got, hx, hy = oracle_mod.bspline_mi(X, Y, bins=nbins, order=order)
    want, whx, why = mi_independent(X, Y, nbins, order)
    np.testing.assert_allclose(hx, whx, rtol=0, atol=1e-10)
    np.testing.assert_allclose(hy, why, rtol=0, atol=1e-10)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-10)


def test_order1_is_histogram_mi(oracle_mod):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(400).astype(np.float32)
    y = (x + 0.5 * rng.standard_normal(400)).astype(np.float32)
    got, _, _ = oracle_mod.bspline_mi(x[None], y[None], bins=6, order=1)
    bx = np.minimum(np.floor(scaled(x, 6, 1)).astype(int), 5)
    by = np.minimum(np.floor(scaled(y, 6, 1)).astype(int), 5)
    joint = np.zeros((6, 6))
    np.add.at(joint, (bx, by), 1.0)
    p = joint / 400
    px, py = p.sum(1), p.sum(0)
    nz = p > 0
    mi = np.sum(p[nz] * np.log2(p[nz] / np.outer(px, py)[nz]))
    assert abs(got[0, 0] - mi) < 1e-12


def test_symmetric_and_self(oracle_mod):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((5, 90)).astype(np.float32)
    mi, hx, _ = oracle_mod.bspline_mi(X, bins=10, order=3)
    np.testing.assert_allclose(mi, mi.T, atol=1e-12)
    assert np.all(np.diag(mi) <= hx + 1e-12)
