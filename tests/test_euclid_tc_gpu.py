"""Euclidean distances on the tensor-core Gram paths against the FP64 oracle,
on the inputs that stress them: clustered points whose distances are tiny
next to their norms (the exact recomputation of near-zero pairs), a single
tight cluster where every pair is recomputed (the per-warp pending queue
fills and drains many times per tile), duplicates, magnitude disparity, and
dimensions that are not a multiple of 4 (scalar recomputation loads).

Error metric: |gpu - oracle| / max(|oracle|, 1e-30) over all pairs (relative,
also for the smallest distances).  Tolerance 4e-6: the split products are
good to ~2^-21 (f16x3) or float32 level (bf16x6), pairs with d^2 below
tau (|a|^2 + |b|^2) are recomputed from the float points, and the square
root is the hardware approximation.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 4e-6


@pytest.fixture(params=["bf16x6", "f16x3"])
def path(request, gpu):
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path(request.param)
    yield request.param
    g.set_gram_path(old)


def run(pts, layout):
    import torch
    import gputools_gb300 as g
    d = g.distances_device(torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda(),
                           "euclidean", layout=layout)
    torch.cuda.synchronize()
    return d.cpu().numpy().astype(np.float64)


def check(pts, oracle_mod, layout):
    n = pts.shape[0]
    got = run(pts, layout)
    want = oracle_mod.dist(pts.astype(np.float32), "euclidean")
    np.fill_diagonal(want, 0.0)
    if layout == "full":
        got = got.reshape(n, n)
    else:
        cols, rows = np.triu_indices(n, 1)
        want = want[cols, rows]
    err = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    err[(want == 0) & (got == 0)] = 0.0
    assert err.max() <= RTOL, (float(err.max()), np.unravel_index(err.argmax(), err.shape))
    return got, want


@pytest.mark.parametrize("layout", ["dist", "full"])
def test_clustered_points(gpu, oracle_mod, path, layout):
    rng = np.random.default_rng(11)
    centres = rng.standard_normal((7, 48)) * 3
    pts = centres[rng.integers(0, 7, 700)] + 1e-3 * rng.standard_normal((700, 48))
    pts[400:420] = pts[10:30]  # exact duplicates
    got, want = check(pts, oracle_mod, layout)
    n = pts.shape[0]
    if layout == "full":
        assert np.all(got.reshape(n, n)[400:420, :][np.arange(20), np.arange(10, 30)] == 0.0)


def test_single_tight_cluster_every_pair_recomputed(gpu, oracle_mod, path):
    rng = np.random.default_rng(12)
    pts = 5.0 + 1e-4 * rng.standard_normal((600, 32))
    check(pts, oracle_mod, "dist")


def test_magnitude_disparity(gpu, oracle_mod, path):
    rng = np.random.default_rng(13)
    pts = rng.standard_normal((300, 24))
    pts[:150] *= 1e-6
    pts[150:] *= 1e6
    check(pts, oracle_mod, "dist")


@pytest.mark.parametrize("dim", [1, 13, 130])
def test_dims_not_multiple_of_four(gpu, oracle_mod, path, dim):
    rng = np.random.default_rng(14 + dim)
    centres = rng.standard_normal((4, dim))
    pts = centres[rng.integers(0, 4, 420)] + 1e-3 * rng.standard_normal((420, dim))
    check(pts, oracle_mod, "full")


def test_random_points_many_tiles(gpu, oracle_mod, path):
    rng = np.random.default_rng(15)
    pts = rng.standard_normal((1300, 64)) * 2 + 1
    check(pts, oracle_mod, "dist")
