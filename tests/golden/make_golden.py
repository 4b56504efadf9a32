"""Generate tests/golden/reference_cpu.npz from the reference's own CPU code.

Runs only where the reference tree is present: oracle/build_ref.sh compiles
src/distance.cpp and src/correlation.cpp from that tree into
oracle/_ref/libref_cpu.so, and this script records seeded inputs with the
outputs of

* distance_host    (src/distance.cpp:174-207; float32 loops of the six metrics)
* permHostKendall  (src/correlation.cpp:506-516; tau-a variant, float counts)
* hostSignif       (src/correlation.cpp:51-64; t-scores with the 0.999 rule)

The fixture lets tests pin the FP64 oracle on machines without the reference.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

OUT = os.path.join(HERE, "reference_cpu.npz")


def main() -> None:
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference CPU build unavailable; nothing generated")
    rng = np.random.default_rng(20240601)
    fx = {}
    # Distances: gpuDist's documented example shape (man/gpuDist.Rd:33-41,
    # 5 x 10 runif) and a ragged N(0,1) case; binary on 0/1 data.
    cases = {
        "runif_5x10": rng.random((5, 10)).astype(np.float32),
        "normal_37x13": rng.standard_normal((37, 13)).astype(np.float32),
        "bern_29x21": (rng.random((29, 21)) < 0.3).astype(np.float32),
    }
    for cname, pts in cases.items():
        fx[f"dist/{cname}/points"] = pts
        for m in oracle.METHODS:
            if m == "canberra" and (pts == 0).any():
                continue  # the reference and R differ on 0/0 terms by design
            for p in ((3.0, 4.0) if m == "minkowski" else (2.0,)):
                key = f"dist/{cname}/{m}/p{p:g}"
                fx[key] = oracle.ref_distance_host(pts, m, p)
    # Kendall without ties: tau-a of the reference equals tau-b.
    X = rng.standard_normal((6, 40)).astype(np.float32)
    Y = rng.standard_normal((4, 40)).astype(np.float32)
    fx["kendall/X"] = X
    fx["kendall/Y"] = Y
    fx["kendall/tau"] = oracle.ref_host_kendall(X, Y)
    # t-scores, including the r >= 0.999 sentinel.
    r = np.concatenate([rng.uniform(-0.99, 0.99, 50), [0.999, 0.9995, 1.0, 0.0]]).astype(np.float32)
    pairs = rng.integers(3, 500, r.size).astype(np.float32)
    fx["signif/r"] = r
    fx["signif/pairs"] = pairs
    fx["signif/ts"] = oracle.ref_host_signif(pairs, r)
    np.savez_compressed(OUT, **fx)
    print(f"wrote {OUT} ({len(fx)} arrays)")


if __name__ == "__main__":
    main()
