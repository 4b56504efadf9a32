"""Pins the FP64 oracle to what the reference's own GPU path returns (CPU only).

tests/golden/reference_gpu.npz holds seeded inputs and the outputs of the
reference's host functions and kernels run on a GB300 by
tests/golden/make_golden_gpu.py (pmcc, bSplineMutualInfo, hcluster,
distance, masterKendall from src/*.cpp with inst/cuda/*.cu, built from the
reference's sources by oracle/build_ref_gpu.sh).  The reference computes in
float32 with --use_fast_math, so the oracle (FP64) is held to it at float
tolerance; counts, NaN patterns and merge orders must be identical.

Where the two differ by design the test says so: the reference's Kendall
kernel (inst/cuda/kendall.cu:18-25, :40-46) counts pairs tied in both
variables as concordant and divides by n(n-1)/2, which is not R's tau-b; the
oracle restates R, and the test checks the reference's own formula from
exact counts instead, and that both agree when there are no ties.
"""
import os

import numpy as np
import pytest

FX = os.path.join(os.path.dirname(__file__), "golden", "reference_gpu.npz")

HC_METHODS = ("single", "complete", "wpgma", "average", "median", "centroid",
              "flexible_group", "flexible", "ward", "mcquitty")


@pytest.fixture(scope="module")
def fx():
    return np.load(FX)


def test_pearson_everything_matches_reference_gpu(oracle_mod, fx):
    x = fx["pe_x"]
    wc, wp, _ = oracle_mod.pearson(x, x.copy(), use=0)
    assert np.abs(fx["pe_corr"] - wc).max() < 2e-6
    assert np.array_equal(fx["pe_pairs"], wp.astype(np.float32))
    # hostSignif (src/correlation.cpp:51-64) on the reference's own r
    rule = oracle_mod.signif(fx["pe_pairs"].astype(np.float64), fx["pe_corr"].astype(np.float64))
    np.testing.assert_allclose(fx["pe_ts"], rule, rtol=1e-5, atol=1e-6)
    wc, wp, _ = oracle_mod.pearson(fx["pe2_a"], fx["pe2_b"], use=0)
    assert np.abs(fx["pe2_corr"] - wc).max() < 2e-6
    assert np.array_equal(fx["pe2_pairs"], wp.astype(np.float32))


def test_pearson_precision_distribution_matches_reference_gpu(oracle_mod, fx):
    """4096 lognormal(5, 1) + offset observations: the reference's float32
    per-pair means and sums stay within 1e-6 of the oracle here."""
    x = fx["pl_x"]
    wc, _, _ = oracle_mod.pearson(x, x.copy(), use=0)
    assert np.abs(fx["pl_corr"] - wc).max() < 1e-6


def test_pearson_pairwise_matches_reference_gpu(oracle_mod, fx):
    wc, wp, wt = oracle_mod.pearson(fx["pp_a"], fx["pp_b"], use=1)
    assert np.array_equal(fx["pp_pairs"], wp.astype(np.float32))
    assert np.array_equal(np.isnan(fx["pp_corr"]), np.isnan(wc))
    ok = ~np.isnan(wc)
    assert np.abs(fx["pp_corr"][ok] - wc[ok]).max() < 2e-6


@pytest.mark.parametrize("tag", ["m1", "m2", "m3"])
def test_mutual_information_matches_reference_gpu(oracle_mod, fx, tag):
    x = fx[f"{tag}_x"]
    wm, _, _ = oracle_mod.bspline_mi(x, bins=int(fx[f"{tag}_bins"]), order=int(fx[f"{tag}_order"]))
    got = fx[f"{tag}_mi"]
    assert np.abs(got - wm).max() < 1e-5 * max(1.0, np.abs(wm).max())


@pytest.mark.parametrize("method", HC_METHODS)
def test_hclust_matches_reference_gpu(oracle_mod, fx, method):
    """Same merges in the same order; heights to float rounding (the
    reference's kernels are compiled with fast math)."""
    sub, sup, hv = oracle_mod.hclust(fx["hc_D"], method)
    assert np.array_equal(sub, fx[f"hc_{method}_sub"])
    assert np.array_equal(sup, fx[f"hc_{method}_sup"])
    rv = fx[f"hc_{method}_val"]
    assert np.max(np.abs(hv - rv) / np.maximum(np.abs(rv), 1e-6)) < 2e-6


@pytest.mark.parametrize("method", ["euclidean", "maximum", "manhattan", "canberra", "binary",
                                    "minkowski"])
def test_distances_match_reference_gpu(oracle_mod, fx, method):
    P = fx["di_Pb"] if method == "binary" else fx["di_P"]
    want = oracle_mod.dist(P, method, 3.0)
    got = fx[f"di_{method}"]
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-6)) < 2e-6


def _reference_kendall_formula(X):
    """inst/cuda/kendall.cu:18-46 from exact counts: C' = concordant pairs plus
    pairs tied in both, tau = (C' - (T - C')) / T with T = n(n-1)/2."""
    X = X.astype(np.float64)
    p, n = X.shape
    iu, ju = np.triu_indices(n, 1)
    sg = np.sign(X[:, ju] - X[:, iu])  # (p, pairs)
    T = n * (n - 1) / 2
    out = np.empty((p, p))
    for a in range(p):
        conc = ((sg[a] * sg) > 0).sum(1) + ((sg[a] == 0) & (sg == 0)).sum(1)
        out[:, a] = (conc - (T - conc)) / T
    return out


def test_kendall_reference_formula_with_ties(oracle_mod, fx):
    x = fx["kt_x"]
    want = _reference_kendall_formula(x)
    np.testing.assert_allclose(fx["kt_tau"], want, rtol=0, atol=1e-6)
    # R's tau-b (what the oracle and the library compute) differs with ties
    tau_b, *_ = oracle_mod.kendall(x)
    assert np.abs(tau_b - fx["kt_tau"]).max() > 1e-2


def test_kendall_without_ties_is_tau_b(oracle_mod, fx):
    x = fx["kc_x"]
    tau_b, *_ = oracle_mod.kendall(x, x.copy(), same=False)
    np.testing.assert_allclose(fx["kc_tau"], tau_b, rtol=0, atol=1e-6)
