"""gt_pmcc_device_noalloc: Pearson without any device allocation.

Callers whose device memory is managed by someone else (a framework's
caching allocator, a fixed memory budget) or who cannot pay for the
synchronisation an allocation can cause use this entry point; its scratch is
a fixed 64 MiB array in the library.  These tests call it through the C ABI
twice in a row and hold each result to the FP64 oracle, within the FP32
tolerance of the Pearson tests (absolute error of r); they cover both `use`
modes, cor(x), two sets of equal size in distinct buffers, the largest
problem whose scratch still fits (checked on sampled rows, the last rows
included), and the rejection of oversized problems.  The file sorts last so a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH = 64 << 20


def tol(n):
    return 2e-6 * np.sqrt(n / 100.0) + 1e-6  # FP32 path tolerance of the Pearson tests


def scratch_bytes(nA, nB, n, sym):
    """The entry point's scratch need: normalised rows and 24-byte column
    statistics of each operand, each part rounded up to 256 bytes."""
    r256 = lambda b: (b + 255) // 256 * 256
    ldz = (n + 3) // 4 * 4
    need = r256(nA * ldz * 4) + r256(nA * 24)
    if not sym:
        need += r256(nB * ldz * 4) + r256(nB * 24)
    return need


def _call(lib, use, dA, dB, nA, nB, n):
    import torch
    out = {k: torch.full((nA, nB), -3.0, dtype=torch.float32, device="cuda")
           for k in ("pairs", "corr", "ts")}
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.gt_pmcc_device_noalloc(use, vp(dA), nA, vp(dB), nB, n, vp(out["pairs"]),
                                    vp(out["corr"]), vp(out["ts"]),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.gt_last_error().decode()
    torch.cuda.synchronize()
    return out


def _check(out, A, B, use, n, oracle_mod, rows=None):
    """Holds corr and pairs (all rows, or the sampled `rows`) to the oracle and
    the t-scores to hostSignif's rule applied to the returned r."""
    if rows is None:
        corr = out["corr"].cpu().numpy()
        pairs = out["pairs"].cpu().numpy()
        ts = out["ts"].cpu().numpy()
        wc, wp, _ = oracle_mod.pearson(A, B, use=use)
    else:
        import torch
        idx = torch.as_tensor(rows, device="cuda")
        corr = out["corr"][idx].cpu().numpy()
        pairs = out["pairs"][idx].cpu().numpy()
        ts = out["ts"][idx].cpu().numpy()
        wc, wp, _ = oracle_mod.pearson(A[rows], B, use=use)
    assert np.array_equal(pairs, wp.astype(np.float32))
    assert np.array_equal(np.isnan(corr), np.isnan(wc))
    ok = ~np.isnan(wc)
    assert np.abs(corr[ok].astype(np.float64) - wc[ok]).max() <= tol(n)
    r = corr.astype(np.float32)
    rule = np.where(r >= np.float32(0.999), np.float32(10000),
                    r * np.sqrt((pairs - np.float32(2)) / (np.float32(1) - r * r)))
    good = ~np.isnan(rule)
    np.testing.assert_allclose(ts[good], rule[good], rtol=2e-6, atol=1e-6)


@pytest.mark.parametrize("use", [0, 1])
@pytest.mark.parametrize("layout", ["same", "distinct", "distinct_equal"])
def test_noalloc_matches_oracle_twice(gpu, oracle_mod, use, layout):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    rng = np.random.default_rng(99 + use + 2 * len(layout))
    n = 257
    A = rng.standard_normal((300, n)).astype(np.float32)
    nb = 300 if layout == "distinct_equal" else 130
    B = (rng.standard_normal((nb, n)) * 3 + 7).astype(np.float32)
    if use == 1:
        A[rng.random(A.shape) < 0.1] = np.nan
        B[rng.random(B.shape) < 0.1] = np.nan
    A[4] = 2.5  # a constant variable: NaN in both modes
    dA = torch.from_numpy(A).cuda()
    if layout == "same":
        B, dB = A, dA
    else:
        dB = torch.from_numpy(B).cuda()
    for _ in range(2):  # the second call reuses the shared array
        out = _call(lib, use, dA, dB, A.shape[0], B.shape[0], n)
        _check(out, A, B, use, n, oracle_mod)


@pytest.mark.parametrize("sym", [True, False])
def test_noalloc_largest_problem_that_fits(gpu, oracle_mod, sym):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    n = 4096
    nA = 1
    while scratch_bytes(nA + 1, nA + 1, n, sym) <= SCRATCH:
        nA += 1
    assert scratch_bytes(nA, nA, n, sym) <= SCRATCH < scratch_bytes(nA + 1, nA + 1, n, sym)
    rng = np.random.default_rng(7 + sym)
    A = (rng.lognormal(5.0, 1.0, (nA, n)) + rng.uniform(0, 1e3, (nA, 1))).astype(np.float32)
    dA = torch.from_numpy(A).cuda()
    if sym:
        B, dB = A, dA
    else:
        B = rng.standard_normal((nA, n)).astype(np.float32)
        B[-1] = A[-1] * 0.5 + B[-1]
        dB = torch.from_numpy(B).cuda()
    rows = np.array([0, 1, nA // 2, nA - 2, nA - 1])
    for _ in range(2):
        out = _call(lib, 0, dA, dB, nA, nA, n)
        _check(out, A, B, 0, n, oracle_mod, rows=rows)
        if sym:
            c = out["corr"]
            assert torch.equal(c, c.T)
    # one more variable on each side no longer fits: rejected before any launch
    # (the 1 x 1 output buffer is never written)
    big = torch.zeros((nA + 1, n), dtype=torch.float32, device="cuda")
    big2 = big if sym else torch.zeros((nA + 1, n), dtype=torch.float32, device="cuda")
    o = torch.empty((1, 1), dtype=torch.float32, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.gt_pmcc_device_noalloc(0, vp(big), nA + 1, vp(big2), nA + 1, n, vp(o), vp(o), vp(o),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1 and "scratch" in lib.gt_last_error().decode()


def test_noalloc_rejects_problems_beyond_its_scratch(gpu):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    n = 4096
    X = torch.zeros((5000, n), dtype=torch.float32, device="cuda")  # 82 MB of scratch needed
    out = torch.empty((1, 1), dtype=torch.float32, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.gt_pmcc_device_noalloc(0, vp(X), 5000, vp(X), 5000, n, vp(out), vp(out), vp(out), sp)
    assert st == 1
    msg = lib.gt_last_error().decode()
    assert "scratch" in msg and str(SCRATCH) in msg
    # an observation count whose size products would wrap is rejected before any use
    st = lib.gt_pmcc_device_noalloc(0, vp(X), 1, vp(X), 1, 1 << 62, vp(out), vp(out), vp(out), sp)
    assert st == 1 and "scratch" in lib.gt_last_error().decode()
