"""Pins the FP64 oracle (CPU only).

The reference ships no tests or golden vectors, so the oracle is held to
(1) the reference's own CPU loops, through tests/golden/reference_cpu.npz
(generated by tests/golden/make_golden.py from src/distance.cpp and
src/correlation.cpp) and directly through oracle/_ref when it is built, and
(2) independent scipy / numpy implementations of the same R definitions.
"""
import os

import numpy as np
import pytest
import scipy.spatial.distance as sd
import scipy.stats as ss

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_cpu.npz")


def test_golden_distances_match_reference_cpu(oracle_mod):
    fx = np.load(GOLDEN)
    n_checked = 0
    for key in fx.files:
        parts = key.split("/")
        if parts[0] != "dist" or len(parts) != 4:
            continue
        _, case, method, ptag = parts
        pts = fx[f"dist/{case}/points"]
        want = fx[key].astype(np.float64)  # reference: float32 arithmetic
        got = oracle_mod.dist(pts, method, float(ptag[1:]))
        scale = np.maximum(np.abs(got), 1.0)
        assert np.max(np.abs(got - want) / scale) < 2e-6, key
        n_checked += 1
    assert n_checked >= 15


def test_golden_kendall_tau_a_equals_tau_b_without_ties(oracle_mod):
    fx = np.load(GOLDEN)
    tau, S, Tx, Ty = oracle_mod.kendall(fx["kendall/X"], fx["kendall/Y"])
    np.testing.assert_allclose(tau, fx["kendall/tau"], rtol=0, atol=1e-7)
    n = fx["kendall/X"].shape[1]
    assert np.all(Tx == n * (n - 1) // 2) and np.all(Ty == n * (n - 1) // 2)


def test_golden_signif(oracle_mod):
    fx = np.load(GOLDEN)
    r = fx["signif/r"].astype(np.float64)
    got = oracle_mod.signif(fx["signif/pairs"], r)
    want = fx["signif/ts"].astype(np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-5)
    assert np.all(got[r >= np.float32(0.999)] == 10000.0)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle",
                                                    "_ref", "libref_cpu.so")),
                    reason="reference CPU build absent (no reference tree here)")
def test_oracle_vs_reference_cpu_random(oracle_mod, rng):
    for (n, d) in [(1, 3), (2, 1), (17, 5), (64, 64)]:
        pts = rng.standard_normal((n, d)).astype(np.float32)
        for m in ("euclidean", "maximum", "manhattan", "canberra", "minkowski"):
            got = oracle_mod.dist(pts, m, 3.0)
            want = oracle_mod.ref_distance_host(pts, m, 3.0).astype(np.float64)
            assert np.max(np.abs(got - want) / np.maximum(np.abs(got), 1)) < 2e-6, (m, n, d)


@pytest.mark.parametrize("method,smethod,kw", [
    ("euclidean", "euclidean", {}), ("maximum", "chebyshev", {}),
    ("manhattan", "cityblock", {}), ("minkowski", "minkowski", {"p": 3.0}),
    ("minkowski", "minkowski", {"p": 1.5})])
def test_dist_vs_scipy(oracle_mod, rng, method, smethod, kw):
    X = rng.standard_normal((40, 11)).astype(np.float32)
    got = oracle_mod.dist(X, method, kw.get("p", 2.0))
    want = sd.cdist(X.astype(np.float64), X.astype(np.float64), smethod, **kw)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)


def test_binary_is_jaccard_on_bits(oracle_mod, rng):
    B = (rng.random((30, 25)) < 0.3).astype(np.float32) * rng.uniform(0.5, 2, (30, 25)).astype(np.float32)
    got = oracle_mod.dist(B, "binary")
    want = sd.cdist(B != 0, B != 0, "jaccard")
    np.testing.assert_allclose(got, np.nan_to_num(want), atol=1e-15)
    Z = np.zeros((3, 4), np.float32)
    assert np.all(oracle_mod.dist(Z, "binary") == 0.0)  # no bit on: 0 (distance.cu:408-412)


def test_canberra_R_rules(oracle_mod):
    # |a-b| / |a+b|; 0/0 terms omitted and the sum scaled by dim/used.
    a = np.array([[1.0, 0.0, 2.0, 0.0], [3.0, 0.0, -1.0, 0.0]], np.float32)
    d = oracle_mod.dist(a, "canberra")
    terms = [abs(1 - 3) / abs(1 + 3), abs(2 + 1) / abs(2 - 1)]
    assert d[0, 1] == pytest.approx(sum(terms) * 4 / 2, rel=1e-15)
    # a = -b != 0 gives an infinite term
    b = np.array([[1.0, 2.0], [-1.0, 2.0]], np.float32)
    assert np.isinf(oracle_mod.dist(b, "canberra")[0, 1])
    # nothing but 0/0 terms: NaN
    z = np.zeros((2, 3), np.float32)
    assert np.isnan(oracle_mod.dist(z, "canberra")[0, 1])


def test_pearson_vs_numpy(oracle_mod, rng):
    A = rng.standard_normal((12, 50)).astype(np.float32)
    B = (rng.standard_normal((7, 50)) * 3 + 100).astype(np.float32)
    c, p, t = oracle_mod.pearson(A, B)
    full = np.corrcoef(np.vstack([A, B]).astype(np.float64))
    np.testing.assert_allclose(c, full[:12, 12:], atol=1e-14)
    assert np.all(p == 50)
    np.testing.assert_allclose(t, c * np.sqrt(48 / (1 - c * c)), rtol=1e-12)


def test_pearson_everything_nan_and_constant(oracle_mod, rng):
    A = rng.standard_normal((4, 20)).astype(np.float32)
    A[1, 3] = np.nan
    A[2, :] = 5.0
    c, p, _ = oracle_mod.pearson(A)
    assert np.all(np.isnan(c[1])) and np.all(np.isnan(c[:, 1]))
    assert np.all(np.isnan(c[2])) and np.all(np.isnan(c[:, 2]))
    assert np.all(p == 20)


def test_pearson_pairwise_vs_masked_numpy(oracle_mod, rng):
    A = rng.standard_normal((6, 40)).astype(np.float32)
    A[rng.random(A.shape) < 0.15] = np.nan
    c, p, _ = oracle_mod.pearson(A, use=1)
    for i in range(6):
        for j in range(6):
            m = ~np.isnan(A[i]) & ~np.isnan(A[j])
            assert p[i, j] == m.sum()
            want = np.corrcoef(A[i][m].astype(np.float64), A[j][m].astype(np.float64))[0, 1]
            assert c[i, j] == pytest.approx(want, abs=1e-13)


def test_kendall_tau_b_vs_scipy_heavy_ties(oracle_mod, rng):
    X = rng.integers(0, 10, (9, 80)).astype(np.float32)
    Y = rng.integers(0, 4, (5, 80)).astype(np.float32)
    tau, S, Tx, Ty = oracle_mod.kendall(X, Y)
    for y in range(5):
        for x in range(9):
            want = ss.kendalltau(X[x].astype(np.float64), Y[y].astype(np.float64)).statistic
            assert tau[y, x] == pytest.approx(want, abs=2e-16)


def test_kendall_exact_counts_bruteforce(oracle_mod, rng):
    X = rng.integers(0, 3, (3, 25)).astype(np.float32)
    tau, S, Tx, Ty = oracle_mod.kendall(X)
    for a in range(3):
        for b in range(3):
            s = tx = ty = 0
            for i in range(25):
                for j in range(i + 1, 25):
                    u = np.sign(X[a, j] - X[a, i]); v = np.sign(X[b, j] - X[b, i])
                    s += u * v; tx += u * u; ty += v * v
            assert (S[b, a], Tx[b, a], Ty[b, a]) == (s, tx, ty)
    assert np.all(np.diag(tau) == 1.0)


def test_kendall_constant_variable_is_nan(oracle_mod):
    X = np.array([[1, 2, 3, 4], [7, 7, 7, 7]], np.float32)
    tau, *_ = oracle_mod.kendall(X, X, same=False)
    assert np.isnan(tau[1, 0]) and np.isnan(tau[0, 1]) and tau[0, 0] == 1.0


def test_ttest_formula(oracle_mod):
    r = np.array([0.5, -0.2, 0.0]); n = np.array([10.0, 30.0, 5.0])
    np.testing.assert_allclose(oracle_mod.ttest(n, r), r * np.sqrt((n - 2) / (1 - r * r)))
