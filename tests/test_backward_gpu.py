"""Adjoint kernels (gpuCorBackward, gpuDistBackward, MDS stress) through the
C ABI against the FP64 oracle adjoints, which tests/test_adjoint_oracle.py
holds to FP64 central finite differences.

Error metric: max |gpu - oracle| / max |oracle| over the gradient.
Tolerances: fp32 and bf16x6 paths 2e-5, bf16x3 2e-4 (its ~2^-16 products),
f16x3 2e-5 (the adjoint GEMM's operand rows are each scaled by a power of
two, then split as f16x3: three products), distance adjoints 2e-5 (float32 CUDA cores up to 64 dimensions;
above, D on the tensor-core distance path and W X as a split-bf16 GEMM).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp32": 2e-5, "bf16x6": 2e-5, "bf16x3": 2e-4, "f16x3": 2e-5}


def rel(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


def cor_bwd_device(lib, X, G):
    import torch
    p, n = X.shape
    dX = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    dG = torch.from_numpy(np.ascontiguousarray(G, np.float32)).cuda()
    out = torch.empty_like(dX)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.gt_cor_backward_device(vp(dX), p, n, vp(dG), vp(out),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.gt_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


@pytest.fixture(params=["fp32", "bf16x3", "bf16x6", "f16x3"])
def path(request, gpu):
    import gputools_gb300 as g
    old = g.get_gram_path()
    g.set_gram_path(request.param)
    yield request.param
    g.set_gram_path(old)


@pytest.mark.parametrize("p,n,sym", [(32, 64, True), (100, 257, False), (300, 1000, True),
                                     (3, 5, False), (2, 7, True), (65, 130, False),
                                     (129, 64, True)])
def test_cor_backward_vs_oracle(gpu, oracle_mod, path, p, n, sym):
    rng = np.random.default_rng(p + n)
    X = (rng.standard_normal((p, n)) * 2 + 10).astype(np.float32)
    G = rng.standard_normal((p, p)).astype(np.float32)
    if sym:
        G = (G + G.T).astype(np.float32)
    got = cor_bwd_device(gpu, X, G)
    want = oracle_mod.cor_backward(X, G.astype(np.float64))
    assert rel(got, want) <= TOL[path], rel(got, want)


def test_cor_backward_single_variable(gpu, path):
    """One variable: C = 1 whatever X is, so the gradient is zero; what the
    kernels return is rounding at the scale |G| / |x - mean| of the terms."""
    rng = np.random.default_rng(4)
    X = (rng.standard_normal((1, 5)) * 3 + 1).astype(np.float32)
    G = np.array([[2.5]], np.float32)
    got = cor_bwd_device(gpu, X, G)
    scale = abs(float(G[0, 0])) / float(np.linalg.norm(X - X.mean()))
    assert np.abs(got).max() <= 1e-5 * scale


def test_cor_backward_constant_variable_has_zero_gradient(gpu, oracle_mod, path):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((20, 50)).astype(np.float32)
    X[4] = 2.5
    G = rng.standard_normal((20, 20)).astype(np.float32)
    got = cor_bwd_device(gpu, X, G)
    assert np.all(got[4] == 0.0)
    want = oracle_mod.cor_backward(X, G.astype(np.float64))
    assert rel(got, want) <= TOL[path]


def test_cor_backward_config_size(gpu, oracle_mod):
    """X 1024 obs x 4096 variables N(0,1), symmetric upstream 4096 x 4096."""
    import gputools_gb300 as g
    rng = np.random.default_rng(11)
    X = rng.standard_normal((4096, 1024)).astype(np.float32)
    G = rng.standard_normal((4096, 4096)).astype(np.float32)
    G = ((G + G.T) * 0.5).astype(np.float32)
    want = oracle_mod.cor_backward(X, G.astype(np.float64))
    for pth in ("bf16x6", "bf16x3", "f16x3"):
        old = g.get_gram_path()
        g.set_gram_path(pth)
        try:
            got = cor_bwd_device(gpu, X, G)
        finally:
            g.set_gram_path(old)
        assert rel(got, want) <= TOL[pth], (pth, rel(got, want))


@pytest.mark.parametrize("n,d", [(1, 3), (33, 7), (300, 32), (257, 64)])
def test_dist_backward_vs_oracle(gpu, oracle_mod, n, d):
    import torch
    rng = np.random.default_rng(n * d)
    X = rng.standard_normal((n, d)).astype(np.float32)
    if n > 10:
        X[5] = X[9]                    # a zero distance: its terms are 0
    G = rng.standard_normal((n, n)).astype(np.float32)
    dX = torch.from_numpy(X).cuda(); dG = torch.from_numpy(G).cuda()
    out = torch.empty_like(dX)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = gpu.gt_dist_backward_device(vp(dX), n, d, vp(dG), vp(out),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, gpu.gt_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    want = oracle_mod.dist_backward(X, G.astype(np.float64))
    if n == 1:
        assert np.all(got == 0)
    else:
        assert rel(got, want) <= 2e-5, rel(got, want)


@pytest.mark.parametrize("n,d", [(64, 32), (1000, 32), (8192, 32), (5000, 16), (3, 8), (701, 13)])
def test_mds_stress_vs_oracle(gpu, oracle_mod, n, d):
    import gputools_gb300 as g
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, d)).astype(np.float32)
    T = rng.standard_normal((n, d)).astype(np.float32)   # seeded 32-dim target embedding
    dT = oracle_mod.dist(T, "euclidean")
    cols, rows = np.triu_indices(n, 1)
    delta = dT[cols, rows].astype(np.float32)
    L, grad = g.gpuMdsStress(X, delta)
    wL, wgrad = oracle_mod.mds_stress(X, delta)
    assert L == pytest.approx(wL, rel=1e-5)
    assert rel(grad, wgrad) <= 5e-5, rel(grad, wgrad)


def test_r_style_wrappers(gpu, oracle_mod):
    import gputools_gb300 as g
    rng = np.random.default_rng(3)
    x = rng.standard_normal((64, 32))                     # 64 obs x 32 variables
    G = rng.standard_normal((32, 32))
    got = g.gpuCorBackward(x, G)
    want = oracle_mod.cor_backward(x.T.astype(np.float32), G).T
    assert got.shape == (64, 32) and rel(got, want) <= 2e-4
    pts = rng.standard_normal((64, 32))
    Gd = rng.standard_normal((64, 64))
    got = g.gpuDistBackward(pts, Gd)
    want = oracle_mod.dist_backward(pts.astype(np.float32), Gd)
    assert rel(got, want) <= 2e-5


def _dist_bwd(lib, X, G):
    import torch
    n, d = X.shape
    dX = torch.from_numpy(X).cuda(); dG = torch.from_numpy(G).cuda()
    out = torch.empty_like(dX)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.gt_dist_backward_device(vp(dX), n, d, vp(dG), vp(out),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.gt_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("n,d,offset", [(700, 65, 0.0), (1000, 128, 50.0), (600, 512, 3.0),
                                        (130, 1000, 0.0), (12, 100, 1.0), (8193, 40, 2.0)])
def test_dist_backward_tensor_core_dims(gpu, oracle_mod, n, d, offset):
    """Above 64 dimensions, and above 32 from 8192 points: GEMMs plus the
    rank-1 correction, on points with a
    common offset (the centring keeps the two terms from cancelling) and a
    duplicated point (its zero distances contribute nothing)."""
    rng = np.random.default_rng(n + d)
    X = (rng.standard_normal((n, d)) + offset).astype(np.float32)
    X[5] = X[9]
    G = rng.standard_normal((n, n)).astype(np.float32)
    got = _dist_bwd(gpu, X, G)
    want = oracle_mod.dist_backward(X, G.astype(np.float64))
    assert rel(got, want) <= 2e-5, rel(got, want)


@pytest.mark.parametrize("n,d", [(500, 128), (2048, 200), (8192, 48)])
def test_mds_stress_tensor_core_dims(gpu, oracle_mod, n, d):
    import gputools_gb300 as g
    rng = np.random.default_rng(n + 1)
    X = rng.standard_normal((n, d)).astype(np.float32)
    X[3] = X[4]  # coincident points: in the stress, not in the gradient
    T = rng.standard_normal((n, d)).astype(np.float32)
    dT = oracle_mod.dist(T, "euclidean")
    cols, rows = np.triu_indices(n, 1)
    delta = dT[cols, rows].astype(np.float32)
    L, grad = g.gpuMdsStress(X, delta)
    wL, wgrad = oracle_mod.mds_stress(X, delta)
    assert L == pytest.approx(wL, rel=1e-5)
    assert rel(grad, wgrad) <= 5e-5, rel(grad, wgrad)


def test_mds_stress_coincident_points_fused_path(gpu, oracle_mod):
    """The fused path (200 points x 16 dimensions) counts coincident points in
    the stress, as the oracle does."""
    import gputools_gb300 as g
    rng = np.random.default_rng(77)
    X = rng.standard_normal((200, 16)).astype(np.float32)
    X[10] = X[20]
    X[30] = X[20]
    delta = (rng.random(200 * 199 // 2) * 3 + 0.5).astype(np.float32)
    L, grad = g.gpuMdsStress(X, delta)
    wL, wgrad = oracle_mod.mds_stress(X, delta)
    assert L == pytest.approx(wL, rel=1e-5)
    assert rel(grad, wgrad) <= 5e-5
