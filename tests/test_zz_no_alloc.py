"""gt_pmcc_device_noalloc: Pearson without any device allocation.

Callers whose device memory is managed by someone else (a framework's
caching allocator, a fixed memory budget) or who cannot pay for the
synchronisation an allocation can cause use this entry point; its scratch is
a fixed array in the library.  This test calls it through the C ABI twice in
a row and compares each result with the allocating entry point
gt_pmcc_device on the same CUDA-core path, within the FP32 tolerance of the
Pearson tests (absolute error of r), and checks that oversized problems are
rejected.  The file sorts last so a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6 * np.sqrt(257 / 100.0) + 1e-6  # FP32 path tolerance at n = 257


def _call(lib, fn, use, A, B, n):
    import torch
    nA, nB = A.shape[0], B.shape[0]
    out = {k: torch.full((nA, nB), -3.0, dtype=torch.float32, device="cuda")
           for k in ("pairs", "corr", "ts")}
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = getattr(lib, fn)(use, vp(A), nA, vp(B), nB, n, vp(out["pairs"]), vp(out["corr"]),
                          vp(out["ts"]), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.gt_last_error().decode()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _close(got, want):
    for k in ("pairs", "corr", "ts"):
        g, w = got[k], want[k]
        assert np.array_equal(np.isnan(g), np.isnan(w)), k
        ok = ~np.isnan(w)
        if k == "pairs":
            assert np.array_equal(g[ok], w[ok])
        elif k == "corr":
            assert np.abs(g[ok] - w[ok]).max() <= TOL
        else:
            small = ok & (np.abs(want["corr"]) < 0.95)
            np.testing.assert_allclose(g[small], w[small], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("use", [0, 1])
@pytest.mark.parametrize("same", [True, False])
def test_noalloc_matches_allocating_entry_point(gpu, use, same):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    rng = np.random.default_rng(99 + use + 2 * same)
    n = 257
    A = rng.standard_normal((300, n)).astype(np.float32)
    B = (rng.standard_normal((130, n)) * 3 + 7).astype(np.float32)
    if use == 1:
        A[rng.random(A.shape) < 0.1] = np.nan
        B[rng.random(B.shape) < 0.1] = np.nan
    dA = torch.from_numpy(A).cuda()
    dB = dA if same else torch.from_numpy(B).cuda()
    old = g.get_gram_path()
    g.set_gram_path("fp32")
    try:
        want = _call(lib, "gt_pmcc_device", use, dA, dB, n)
    finally:
        g.set_gram_path(old)
    first = _call(lib, "gt_pmcc_device_noalloc", use, dA, dB, n)
    second = _call(lib, "gt_pmcc_device_noalloc", use, dA, dB, n)
    _close(first, want)
    _close(second, want)


def test_noalloc_rejects_problems_beyond_its_scratch(gpu):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    n = 4096
    X = torch.zeros((5000, n), dtype=torch.float32, device="cuda")  # 82 MB of scratch needed
    out = torch.empty((1, 1), dtype=torch.float32, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.gt_pmcc_device_noalloc(0, vp(X), 5000, vp(X), 5000, n, vp(out), vp(out), vp(out),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1
    msg = lib.gt_last_error().decode()
    assert "scratch" in msg and str(64 << 20) in msg
