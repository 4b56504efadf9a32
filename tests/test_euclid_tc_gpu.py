"""Euclidean distances on the tensor-core Gram paths against the FP64 oracle,
on the inputs that stress them: clustered points whose distances are tiny
next to their norms (the exact recomputation of near-zero pairs), a single
tight cluster where every pair is recomputed (the per-warp pending queue
fills and drains many times per tile), duplicates, magnitude disparity, and
dimensions that are not a multiple of 4 (scalar recomputation loads).

The dist layout runs both tilings: the triangular one and the aligned-line
one (a permuted column operand so that every warp store is one whole
128-byte line; GT_EUCLID_LINES forces it on or off), including outputs that
start inside a line and sizes that span several 8192-column super-blocks.

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


@pytest.fixture(params=["0", "1"], ids=["tri", "lines"])
def lines(request, monkeypatch):
    monkeypatch.setenv("GT_EUCLID_LINES", request.param)
    return request.param


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
def test_clustered_points(gpu, oracle_mod, path, lines, layout):
    rng = np.random.default_rng(11)
    centres = rng.standard_normal((7, 48)) * 3
    pts = centres[rng.integers(0, 7, 700)] + 1e-3 * rng.standard_normal((700, 48))
    pts[400:420] = pts[10:30]  # exact duplicates
    got, want = check(pts, oracle_mod, layout)
    n = pts.shape[0]
    if layout == "full":
        assert np.all(got.reshape(n, n)[400:420, :][np.arange(20), np.arange(10, 30)] == 0.0)


def test_single_tight_cluster_every_pair_recomputed(gpu, oracle_mod, path, lines):
    rng = np.random.default_rng(12)
    pts = 5.0 + 1e-4 * rng.standard_normal((600, 32))
    check(pts, oracle_mod, "dist")


def test_magnitude_disparity(gpu, oracle_mod, path, lines):
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


def test_random_points_many_tiles(gpu, oracle_mod, path, lines):
    rng = np.random.default_rng(15)
    pts = rng.standard_normal((1300, 64)) * 2 + 1
    check(pts, oracle_mod, "dist")


def dist_base(n, c):
    c = np.asarray(c, np.int64)
    return n * c - c * (c + 1) // 2 - c - 1


@pytest.mark.parametrize("offset", [0, 7, 31])
def test_lines_output_offsets_and_guards(gpu, oracle_mod, path, monkeypatch, offset):
    """Aligned lines with the output starting `offset` floats into a line:
    the classes follow the real address, and nothing outside the dist
    vector is written."""
    import torch
    import gputools_gb300 as g
    monkeypatch.setenv("GT_EUCLID_LINES", "1")
    rng = np.random.default_rng(21 + offset)
    centres = rng.standard_normal((5, 40)) * 2
    pts = centres[rng.integers(0, 5, 1100)] + 1e-3 * rng.standard_normal((1100, 40))
    pts[700:730] = pts[3:33]
    n = pts.shape[0]
    count = n * (n - 1) // 2
    buf = torch.full((count + 64,), -7.0, dtype=torch.float32, device="cuda")
    out = buf[offset:offset + count]
    g.distances_device(torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda(),
                       "euclidean", layout="dist", out=out)
    torch.cuda.synchronize()
    host = buf.cpu().numpy()
    assert np.all(host[:offset] == -7.0) and np.all(host[offset + count:] == -7.0)
    got = host[offset:offset + count].astype(np.float64)
    want = oracle_mod.dist(pts.astype(np.float32), "euclidean")
    cols, rows = np.triu_indices(n, 1)
    want = want[cols, rows]
    err = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    err[(want == 0) & (got == 0)] = 0.0
    assert err.max() <= RTOL, float(err.max())


@pytest.mark.parametrize("n,mode", [(9000, "1"), (17000, "1"), (33000, "")])
def test_lines_super_blocks_sampled(gpu, oracle_mod, path, monkeypatch, n, mode):
    """Sizes that span two to five super-blocks (8192 columns each), forced
    and automatic; every entry of sampled points (super-block edges, the
    first and last points, random ones) against the oracle."""
    import torch
    import gputools_gb300 as g
    monkeypatch.setenv("GT_EUCLID_LINES", mode)
    rng = np.random.default_rng(n)
    centres = rng.standard_normal((9, 24)) * 3
    pts = (centres[rng.integers(0, 9, n)] + 1e-2 * rng.standard_normal((n, 24))).astype(np.float32)
    pts[n - 40:] = pts[100:140]  # duplicates across super-blocks
    d = g.distances_device(torch.from_numpy(pts).cuda(), "euclidean", layout="dist")
    samples = np.unique(np.concatenate([[0, 1, 2, n - 2, n - 1, 8191, 8192, 8193, 16383, 16384,
                                         n // 2], rng.integers(0, n, 9)]))
    samples = samples[samples < n]
    want = oracle_mod.dist(pts, "euclidean", 2.0, b=pts[samples])  # [k, x] = d(x, samples[k])
    xs = np.arange(n, dtype=np.int64)
    for k, s in enumerate(samples):
        other = xs[xs != s]
        idx = np.where(other < s, dist_base(n, other) + s, dist_base(n, s) + other)
        got = d[torch.from_numpy(idx).cuda()].cpu().numpy().astype(np.float64)
        w = want[k, other]
        err = np.abs(got - w) / np.maximum(np.abs(w), 1e-30)
        err[(w == 0) & (got == 0)] = 0.0
        assert err.max() <= RTOL, (int(s), float(err.max()), int(other[err.argmax()]))


def test_lines_pair_list_overflow(gpu, oracle_mod, path, monkeypatch):
    """A single tight cluster of 12000 points: every pair is recomputed, more
    than a warp's region of the pair list holds, so the epilogue warps also
    recompute pairs themselves; sampled points against the oracle."""
    import torch
    import gputools_gb300 as g
    monkeypatch.setenv("GT_EUCLID_LINES", "1")
    rng = np.random.default_rng(31)
    n = 12000
    pts = (3.0 + 1e-4 * rng.standard_normal((n, 16))).astype(np.float32)
    d = g.distances_device(torch.from_numpy(pts).cuda(), "euclidean", layout="dist")
    samples = np.unique(np.concatenate([[0, 1, n - 1, 8191, 8192], rng.integers(0, n, 7)]))
    want = oracle_mod.dist(pts, "euclidean", 2.0, b=pts[samples])
    xs = np.arange(n, dtype=np.int64)
    for k, s in enumerate(samples):
        other = xs[xs != s]
        idx = np.where(other < s, dist_base(n, other) + s, dist_base(n, s) + other)
        got = d[torch.from_numpy(idx).cuda()].cpu().numpy().astype(np.float64)
        w = want[k, other]
        err = np.abs(got - w) / np.maximum(np.abs(w), 1e-30)
        err[(w == 0) & (got == 0)] = 0.0
        assert err.max() <= RTOL, (int(s), float(err.max()), int(other[err.argmax()]))
