"""Batched problems (one plan, replayed from a CUDA graph) against the
single-problem C ABI paths and the oracle.

Pearson: absolute error of r within the tolerance of the Pearson tests for
the Gram path (bf16x3 2e-5; bf16x6 and f16x3 2e-6 * sqrt(n / 100) + 1e-6) of
the oracle, and equal to the single-problem tensor-core result to 1e-6.
Kendall: bit-exact against the oracle's tau-b.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shapes(rng, count, pmax, nmin, nmax):
    p = np.exp(rng.uniform(np.log(1), np.log(pmax), count)).astype(int)
    n = np.exp(rng.uniform(np.log(nmin), np.log(nmax), count)).astype(int)
    return list(zip(p.tolist(), n.tolist()))


def _tol(path, n):
    return 2e-5 if path == "bf16x3" else 2e-6 * np.sqrt(max(n, 1) / 100.0) + 1e-6


@pytest.fixture
def gram_path(request):
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path(request.param)
    yield request.param
    g.set_gram_path(old)


@pytest.mark.parametrize("gram_path,graph", [("bf16x3", True), ("bf16x3", False),
                                             ("bf16x6", True), ("f16x3", True),
                                             ("f16x3", False)], indirect=["gram_path"])
def test_pearson_batch_matches_single_and_oracle(gpu, oracle_mod, gram_path, graph):
    import torch
    import gputools_gb300 as g
    rng = np.random.default_rng(31)
    # p of every residue mod 8 (row strides off the 32-byte sectors) and
    # problems of several tile rows and columns
    shapes = _shapes(rng, 40, 600, 3, 900) + [(1, 10), (128, 64), (257, 129), (300, 2),
                                              (1023, 70), (777, 300), (520, 33)]
    xs = [rng.standard_normal((p, n)).astype(np.float32) * 2 + 5 for p, n in shapes]
    dxs = [torch.from_numpy(x).cuda() for x in xs]
    with g.BatchPlan(dxs, "pearson", graph=graph) as plan:
        assert gram_path in plan.describe()
        outs = plan.launch()
        torch.cuda.synchronize()
        for x, dx, o in zip(xs, dxs, outs):
            corr = o["corr"].cpu().numpy()
            want, wp, _ = oracle_mod.pearson(x)
            ok = ~np.isnan(want)
            assert np.array_equal(np.isnan(corr), np.isnan(want))
            if ok.any():
                assert np.abs(corr[ok] - want[ok]).max() <= _tol(gram_path, x.shape[1])
            assert np.all(o["pairs"].cpu().numpy() == x.shape[1])
            # t-scores in both orientations: hostSignif's rule on the stored r
            r = corr.astype(np.float32)
            ts = o["ts"].cpu().numpy()
            rule = np.where(r >= np.float32(0.999), np.float32(10000),
                            r * np.sqrt((np.float32(x.shape[1]) - 2) / (np.float32(1) - r * r)))
            # 1 - r^2 cancels near |r| = 1: there the rounding of r * r (the
            # kernel fuses it) moves t by ~eps / (1 - r^2) relative
            fin = ~np.isnan(rule)
            well = fin & (np.abs(r) < 0.99)
            np.testing.assert_allclose(ts[well], rule[well], rtol=2e-6, atol=1e-6)
            np.testing.assert_allclose(ts[fin], rule[fin], rtol=1e-3, atol=1e-6)
            single = g.pmcc_device(dx)["corr"].cpu().numpy()
            assert np.allclose(corr, single, atol=1e-6, equal_nan=True)


def test_pearson_batch_pitched_outputs(gpu):
    """Pitched outputs (rows a multiple of 8 floats apart) hold the same
    values as contiguous ones and leave the padding columns alone; a stride
    below p is refused."""
    import ctypes
    import torch
    import gputools_gb300 as g
    from gputools_gb300 import _lib
    rng = np.random.default_rng(12)
    xs = [torch.from_numpy(rng.standard_normal((p, 90)).astype(np.float32)).cuda()
          for p in (1, 7, 129, 300, 515)]
    with g.BatchPlan(xs, "pearson", pitched=False) as plain:
        want = [{k: v.clone() for k, v in o.items()} for o in plain.launch()]
    with g.BatchPlan(xs, "pearson") as plan:
        bases = []
        for x, o in zip(xs, plan.outputs):
            p = x.shape[0]
            ld = (p + 7) // 8 * 8
            assert o["corr"].shape == (p, p) and o["corr"].stride() == (ld, 1)
            base = {k: torch.as_strided(v, (p, ld), (ld, 1)) for k, v in o.items()}
            for b in base.values():
                b.fill_(-7.0)
            bases.append(base)
        outs = plan.launch()
        torch.cuda.synchronize()
        for x, o, w, base in zip(xs, outs, want, bases):
            p = x.shape[0]
            for k in ("corr", "ts", "pairs"):
                assert torch.equal(o[k], w[k]) or torch.allclose(o[k], w[k], equal_nan=True, atol=0)
                assert bool((base[k][:, p:] == -7.0).all())
    x = xs[2]
    out = torch.empty((129, 129), device="cuda")
    arr = (_lib.CorProblem * 1)()
    arr[0] = _lib.CorProblem(x.data_ptr(), 129, 90, out.data_ptr(), 0, 0, 100)
    h = ctypes.c_void_p()
    assert g.load().gt_pmcc_batch_plan_create(arr, 1, 0, ctypes.byref(h)) != 0
    assert b"stride" in g.load().gt_last_error()


def test_pearson_batch_replay_sees_new_inputs(gpu, oracle_mod):
    import torch
    import gputools_gb300 as g
    rng = np.random.default_rng(5)
    xs = [torch.from_numpy(rng.standard_normal((p, 200)).astype(np.float32)).cuda()
          for p in (50, 300, 7)]
    with g.BatchPlan(xs, "pearson") as plan:
        plan.launch()
        for x in xs:
            x.copy_(torch.from_numpy(rng.standard_normal(tuple(x.shape)).astype(np.float32)))
        outs = plan.launch()
        torch.cuda.synchronize()
        for x, o in zip(xs, outs):
            want, _, _ = oracle_mod.pearson(x.cpu().numpy())
            assert np.abs(o["corr"].cpu().numpy() - want).max() <= 2e-5


def test_pearson_batch_autotune(gpu, tmp_path, monkeypatch):
    import torch
    import gputools_gb300 as g
    monkeypatch.setenv("GT_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(6)
    xs = [torch.from_numpy(rng.standard_normal((p, 300)).astype(np.float32)).cuda()
          for p in (400, 90, 1000)]
    with g.BatchPlan(xs, "pearson", autotune=True) as plan:
        assert "tuned" in plan.describe()
        plan.launch()
    assert (tmp_path / "tune.txt").exists()


@pytest.mark.parametrize("graph", [True, False])
def test_kendall_batch_bit_exact(gpu, oracle_mod, graph):
    import torch
    import gputools_gb300 as g
    rng = np.random.default_rng(41)
    shapes = [(p, 200) for p, _ in _shapes(rng, 25, 200, 2, 3)] + [(1, 5), (65, 31), (130, 64), (3, 2)]
    xs = [rng.integers(0, 20, (p, n)).astype(np.float32) for p, n in shapes]
    with g.BatchPlan([torch.from_numpy(x).cuda() for x in xs], "kendall", graph=graph) as plan:
        outs = plan.launch()
        torch.cuda.synchronize()
        for x, o in zip(xs, outs):
            want, *_ = oracle_mod.kendall(x)
            got = o.cpu().numpy()
            assert np.array_equal(np.isnan(got), np.isnan(want))
            assert np.array_equal(got[~np.isnan(got)], want[~np.isnan(want)])


def test_batch_rejects_bad_problems(gpu):
    import torch
    import gputools_gb300 as g
    x = torch.zeros((4, 0), dtype=torch.float32, device="cuda")
    with pytest.raises(g.GpuToolsError, match="no observations|null input"):
        g.BatchPlan([x], "pearson")
