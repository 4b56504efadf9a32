"""Record what the reference's own GPU path returns, as test fixtures.

Runs on a host with a CUDA device and the staged reference build
(baseline/_ref/libref_gpu.so, made by oracle/build_ref_gpu.sh from the copy
oracle/stage_ref.sh places there): the reference's host functions pmcc()
(src/correlation.cpp:66-161), bSplineMutualInfo() (src/mi.cpp:33-164),
hcluster() (src/hcluster.cpp:15-38), distance() (src/distance.cpp:259-316)
and masterKendall() (src/kendall.cpp:13-55) with their kernels from
inst/cuda/*.cu, on seeded inputs at the sizes of the small configurations
(500 observations for Pearson, as gpuCor's 500 x 1000 case; 300 samples for
gpuMi; 150 points for the clustering).  Inputs and outputs go to one
compressed .npz (tests/golden/reference_gpu.npz), which tests/test_oracle.py
holds the FP64 oracle to.

Every input is sized inside the reference kernels' limits (grids below 65535
in y, gpuMi with nx == ny, finite values) so that its kernels stay in bounds.

    python tests/golden/make_golden_gpu.py [out.npz]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

HC_METHODS = ("single", "complete", "wpgma", "average", "median", "centroid",
              "flexible_group", "flexible", "ward", "mcquitty")
DIST_METHODS = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")


def main(out_path):
    oracle.build()
    rng = np.random.default_rng(20260)
    rec = {}

    # Pearson, use = "everything": cor(x) through .C (two copies of x) and two sets
    x = (rng.standard_normal((120, 500)) * 2 + 3).astype(np.float32)
    rec["pe_x"] = x
    rec["pe_corr"], rec["pe_pairs"], rec["pe_ts"] = oracle.ref_gpu_pmcc(x, x.copy(), use=0)
    a = rng.standard_normal((60, 500)).astype(np.float32)
    b = (rng.standard_normal((90, 500)) * 0.5 - 7 + 0.3 * np.repeat(a[:30], 3, 0)).astype(np.float32)
    rec["pe2_a"], rec["pe2_b"] = a, b
    rec["pe2_corr"], rec["pe2_pairs"], rec["pe2_ts"] = oracle.ref_gpu_pmcc(a, b, use=0)
    # the precision configuration's distribution (lognormal(5, 1) plus offsets
    # in [0, 1e3]) over its 4096 observations
    xl = (rng.lognormal(5.0, 1.0, (48, 4096)) + rng.uniform(0, 1e3, (48, 1))).astype(np.float32)
    rec["pl_x"] = xl
    rec["pl_corr"], rec["pl_pairs"], _ = oracle.ref_gpu_pmcc(xl, xl.copy(), use=0)
    # use = "pairwise.complete.obs" with missing values
    pa = rng.standard_normal((50, 300)).astype(np.float32)
    pb = (rng.standard_normal((70, 300)) + 4).astype(np.float32)
    pa[rng.random(pa.shape) < 0.10] = np.nan
    pb[rng.random(pb.shape) < 0.05] = np.nan
    rec["pp_a"], rec["pp_b"] = pa, pb
    rec["pp_corr"], rec["pp_pairs"], rec["pp_ts"] = oracle.ref_gpu_pmcc(pa, pb, use=1)

    # gpuMi(x): a shared component so that the MI values spread
    for tag, bins, order in (("m1", 10, 3), ("m2", 2, 1), ("m3", 7, 2)):
        xm = (rng.standard_normal((1, 300)) + 0.8 * rng.standard_normal((80, 300))).astype(np.float32)
        rec[f"{tag}_x"] = xm
        rec[f"{tag}_bins"] = np.int32(bins)
        rec[f"{tag}_order"] = np.int32(order)
        rec[f"{tag}_mi"] = oracle.ref_gpu_mi(xm, bins, order)

    # gpuHclust: euclidean distances of 150 points around 5 centres
    cen = rng.standard_normal((5, 8)) * 3
    pts = (cen[rng.integers(0, 5, 150)] + rng.standard_normal((150, 8))).astype(np.float32)
    D = np.sqrt(((pts[:, None, :].astype(np.float64) - pts[None, :, :]) ** 2).sum(-1)).astype(np.float32)
    rec["hc_D"] = D
    for m in HC_METHODS:
        sub, sup, val = oracle.ref_gpu_hcluster(D, m)
        rec[f"hc_{m}_sub"], rec[f"hc_{m}_sup"], rec[f"hc_{m}_val"] = sub, sup, val

    # gpuDist: all six methods
    P = rng.standard_normal((100, 20)).astype(np.float32)
    Pb = (rng.random((100, 20)) < 0.3).astype(np.float32)
    rec["di_P"], rec["di_Pb"] = P, Pb
    for m in DIST_METHODS:
        pts_m = Pb if m == "binary" else P
        rec[f"di_{m}"] = oracle.ref_gpu_distance(pts_m, m, 3.0)

    # gpuCor(method = "kendall"): heavy ties (integers 0..9) and no ties
    kx = rng.integers(0, 10, (40, 60)).astype(np.float32)
    kc = rng.standard_normal((30, 60)).astype(np.float32)
    rec["kt_x"], rec["kc_x"] = kx, kc
    rec["kt_tau"] = oracle.ref_gpu_kendall(kx, kx.copy())
    rec["kc_tau"] = oracle.ref_gpu_kendall(kc, kc.copy())

    np.savez_compressed(out_path, **rec)
    print(f"wrote {out_path}: {len(rec)} arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "gpurun_out", "reference_gpu.npz"))
