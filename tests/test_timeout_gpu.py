"""The bounded-wait abort path of the tensor-core kernels.

Every mbarrier wait in the tcgen05 kernels has a limit; a wait that gives up
makes its CTA stop issuing work, wait for its in-flight copies and
multiplies, free its tensor memory and set the device's error word.  Here the
limit is set to 2 microseconds (gt_set_wait_limit_ns), short enough that
waits give up while their copies and multiplies are still in flight (nothing
is left that could hang: the copies complete, and the drain waits for them).
The call must then report GT_ETIMEOUT -- through gt_device_status for the
device entry, directly for the host entry -- or GT_OK if every wait happened
to finish in time; with the limit restored, the next call must match the
FP64 oracle, so the context stays usable.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GT_OK, GT_ETIMEOUT = 0, 5


def _data(rng, p, n, nan):
    X = (rng.lognormal(5.0, 1.0, (p, n)) + rng.uniform(0, 1e3, (p, 1))).astype(np.float32)
    if nan:
        X[rng.random(X.shape) < 0.01] = np.nan
    return X


@pytest.mark.parametrize("path,use", [("f16x3", 0), ("f16x6", 0), ("f16x3", 1)])
def test_short_wait_limit_reports_timeout_and_recovers(gpu, oracle_mod, path, use):
    import torch
    import gputools_gb300 as g
    lib = g.load()
    rng = np.random.default_rng(17)
    p, n = 1536, 4096
    X = _data(rng, p, n, nan=use == 1)
    dX = torch.from_numpy(X).cuda()
    out = [torch.empty((p, p), dtype=torch.float32, device="cuda") for _ in range(3)]
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    old = g.get_gram_path()
    g.set_gram_path(path)
    try:
        assert lib.gt_device_status(sp) == GT_OK  # nothing pending from earlier tests
        assert lib.gt_set_wait_limit_ns(2000) == GT_OK
        seen = set()
        for _ in range(3):
            st = lib.gt_pmcc_device(use, vp(dX), p, vp(dX), p, n, vp(out[0]), vp(out[1]),
                                    vp(out[2]), sp)
            assert st == GT_OK, lib.gt_last_error().decode()
            st = lib.gt_device_status(sp)
            assert st in (GT_OK, GT_ETIMEOUT), st
            seen.add(st)
            # the word is cleared by the check
            assert lib.gt_device_status(sp) == GT_OK
        # the host entry reports it itself
        hp = np.empty((p, p), np.float32)
        hc = np.empty((p, p), np.float32)
        ht = np.empty((p, p), np.float32)
        hv = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        st = lib.gt_pmcc(use, hv(X), p, hv(X), p, n, hv(hp), hv(hc), hv(ht))
        assert st in (GT_OK, GT_ETIMEOUT), lib.gt_last_error().decode()
        seen.add(st)
        assert GT_ETIMEOUT in seen, "a 2 us limit never gave up a wait"
    finally:
        lib.gt_set_wait_limit_ns(0)
        g.set_gram_path(old)
    # the default limit again: the same call completes and matches the oracle
    g.set_gram_path(path)
    try:
        st = lib.gt_pmcc_device(use, vp(dX), p, vp(dX), p, n, vp(out[0]), vp(out[1]), vp(out[2]),
                                sp)
        assert st == GT_OK
        assert lib.gt_device_status(sp) == GT_OK
    finally:
        g.set_gram_path(old)
    rows = np.array([0, 7, 511, 1024, p - 1])
    got = out[1][torch.as_tensor(rows, device="cuda")].cpu().numpy().astype(np.float64)
    want, wp, _ = oracle_mod.pearson(X[rows], X, use=use)
    for k, r in enumerate(rows):
        if not np.isnan(want[k, r]):
            want[k, r] = 1.0
    ok = ~np.isnan(want)
    assert np.array_equal(np.isnan(got), ~ok)
    tol = 2e-5 if use == 1 else (1.5e-7 if path == "f16x6" else 2e-6 * np.sqrt(n / 100) + 1e-6)
    assert np.abs(got[ok] - want[ok]).max() <= tol
    assert np.array_equal(out[0][torch.as_tensor(rows, device="cuda")].cpu().numpy(),
                          wp.astype(np.float32))
