#!/usr/bin/env python
"""Benchmark of the all-pairs hot path on GB300.

Headline workload (the configuration the metric is quoted on): gpuCor
pearson, cor(x) of x = 4096 observations x 20000 variables float32, values
lognormal(mu=5, sigma=1) plus per-column offsets uniform in [0, 1e3].  One
step = one full gt_pmcc_device call (FP64 column statistics, tcgen05 Gram
contraction, fused epilogue writing coefficients, t-scores and pair counts
for all 20000^2 entries).  value = entries of the returned matrix per
second, on the Gram path that meets the metric's bar (max relative error
<= 1e-6 against FP64 for |r| >= 0.01): the error-free f16x6 split.  The same
line carries every other Gram path on the same workload (f16x3, bf16x6,
bf16x3, the plain FP32 CUDA-core path) with their errors against the FP64
oracle on sampled rows, the Euclidean precision workload (100000 points x
128 from 1000 clusters, sd 1e-3, 5% exact duplicates, R `dist` layout), the
end-to-end number through the host C ABI with the ordinary (pageable) host
buffers R's .C passes (pinned buffers beside it), the roofline of the Gram
kernel, clocks, the CPU baseline, and -- where the reference's own code is
built on the host -- its GPU path and host loops timed on the same machine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs an independent replica (the path is computed
per GPU, no collective); value sums the ranks' entries over the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Pearson/Euclid entries/s, split-BF16 TC vs FP32 at max rel err ≤1e-6 vs FP64"
N_OBS, N_VARS = 4096, 20000
E_POINTS, E_DIM, E_CLUSTERS, E_SD, E_DUP = 100_000, 128, 1000, 1e-3, 0.05
SAMPLE_ROWS = 48


# ----------------------------------------------------------------------------- helpers

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Ranks:
    """One process per GPU under torchrun (NCCL); "gloo" runs the same barrier
    and max-over-ranks on CPU tensors (the multi-process tests)."""

    def __init__(self, backend: str = "nccl"):
        self.world, self.rank, self.local = dist_env()
        self.dist = None
        self.device = "cuda" if backend == "nccl" else "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if not self.dist:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class Clocks:
    """nvidia-smi sampling while the timed regions run."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            out["reasons"] = ["nvidia-smi unavailable"]
            return out
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return out
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v == "Active"})
        load = [r for r in rows if r[2] > 250.0] or rows
        out.update(sm_mhz=float(np.median([r[0] for r in load])), sm_max_mhz=max(r[1] for r in rows),
                   reasons=reasons, samples=len(rows))
        return out


def make_pearson_data(seed: int = 3) -> np.ndarray:
    """(N_VARS, N_OBS) float32, variable-major (R's as.single(x) order)."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((N_VARS, N_OBS), dtype=np.float32)
    x = np.exp(z + np.float32(5.0), dtype=np.float32)
    x += rng.uniform(0.0, 1e3, (N_VARS, 1)).astype(np.float32)
    return x


def make_euclid_data(seed: int = 4) -> np.ndarray:
    """(E_POINTS, E_DIM) float32 from E_CLUSTERS Gaussian clusters (sd E_SD)
    with E_DUP of the points exact copies of other points."""
    rng = np.random.default_rng(seed)
    centres = rng.standard_normal((E_CLUSTERS, E_DIM), dtype=np.float32)
    lab = rng.integers(0, E_CLUSTERS, E_POINTS)
    pts = centres[lab] + np.float32(E_SD) * rng.standard_normal((E_POINTS, E_DIM), dtype=np.float32)
    ndup = int(E_DUP * E_POINTS)
    dst = rng.choice(E_POINTS, ndup, replace=False)
    src = rng.integers(0, E_POINTS, ndup)
    pts[dst] = pts[src]
    return np.ascontiguousarray(pts, dtype=np.float32)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


# ----------------------------------------------------------------------------- reference arm

def run_reference(args, ranks: Ranks):
    """The reference's CPU implementation of the path (the FP64 oracle port;
    the reference's own compiled loops cannot run on the GPU hosts) on bounded
    samples of the headline workload, all host threads."""
    if ranks.rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    X = make_pearson_data()
    rows_per_step = 8
    rng = np.random.default_rng(11)
    for _ in range(args.warmup):
        r = rng.choice(N_VARS, rows_per_step, replace=False)
        oracle.pearson(X[r], X)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = rng.choice(N_VARS, rows_per_step, replace=False)
        oracle.pearson(X[r], X)
    dt = (time.perf_counter() - t0) / args.steps
    value = rows_per_step * N_VARS / dt
    sample = f"{rows_per_step} rows x {N_VARS} variables x {N_OBS} obs per step (FP64 oracle port)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "entries/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"gpuCor pearson {N_OBS} obs x {N_VARS} vars, cor(x), everything",
                   "sample": sample},
        "cpu_baseline": {"value": value, "unit": "entries/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "entries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- our arm

def run_ours(args, ranks: Ranks):
    import torch
    import gputools_gb300 as g
    from gputools_gb300 import _lib

    torch.cuda.set_device(ranks.local)
    lib = g.load()
    dev = torch.device("cuda", ranks.local)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    peaks, peaks_kind = load_peaks()

    X = make_pearson_data()
    dX = torch.from_numpy(X).to(dev)
    P = N_VARS
    corr = torch.empty((P, P), dtype=torch.float32, device=dev)
    ts = torch.empty_like(corr)
    pairs = torch.empty_like(corr)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())

    def pearson_step():
        _lib.check(lib.gt_pmcc_device(0, vp(dX), P, vp(dX), P, N_OBS, vp(pairs), vp(corr), vp(ts),
                                      sptr))

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ranks.barrier()
        torch.cuda.synchronize()
        l0 = lib.gt_kernel_launches()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ranks.barrier()
        ms = e0.elapsed_time(e1) / steps
        return ranks.max(ms), lib.gt_kernel_launches() - l0

    # headline path: the error-free fixed-point split (f16x6: relative error of
    # r <= 1e-6 against FP64 for |r| >= 0.01, the metric's bar), unless the
    # tensor-core path is unavailable
    headline = "f16x6"
    try:
        g.set_gram_path(headline)
        pearson_step()
        torch.cuda.synchronize()
    except _lib.GpuToolsError:
        headline = "fp32"
        g.set_gram_path(headline)

    clocks = Clocks(ranks.local)
    clocks.start()
    lib.gt_profile_reset()
    lib.gt_profile_enable(1)
    ms, launches = timed(pearson_step, args.steps, args.warmup)
    lib.gt_profile_enable(0)
    gram_ms = ctypes.c_double(0)
    gram_n = ctypes.c_uint64(0)
    lib.gt_profile_kernel_ms(b"pearson_gram", ctypes.byref(gram_ms), ctypes.byref(gram_n))
    entries = float(P) * P
    value = ranks.world * entries / (ms * 1e-3)

    # precision on sampled rows against the FP64 oracle
    import oracle
    oracle.build()
    rng = np.random.default_rng(7)
    rows = np.sort(rng.choice(P, SAMPLE_ROWS, replace=False))

    t_cpu0 = time.perf_counter()
    want_rows, _, _ = oracle.pearson(X[rows], X)
    cpu_dt = time.perf_counter() - t_cpu0  # the oracle on SAMPLE_ROWS rows
    for k, r in enumerate(rows):
        want_rows[k, r] = 1.0

    def max_err(c):
        """max |dr|, and max |dr| / |r| over the entries with |r| >= 0.1 and >= 0.01"""
        got = c[torch.from_numpy(rows).to(dev)].cpu().numpy().astype(np.float64)
        d = np.abs(got - want_rows)
        res = {"max_abs_err": float(d.max())}
        for floor in (0.1, 0.01):
            big = np.abs(want_rows) >= floor
            res[f"max_rel_err_r_ge_{floor}"] = float((d[big] / np.abs(want_rows[big])).max())
        return res

    head_err = max_err(corr)

    # the other Gram paths on the same workload (rank 0 only; extras)
    paths = {}
    if ranks.rank == 0:
        for pth in ("f16x6", "f16x3", "bf16x6", "bf16x3", "fp32"):
            if pth == headline:
                paths[pth] = {"entries_per_s": value / ranks.world, "ms_per_step": ms,
                              "gram_ms": gram_ms.value / max(1, gram_n.value), **head_err}
                continue
            try:
                g.set_gram_path(pth)
                k = max(3, args.steps // 4)
                lib.gt_profile_reset()
                lib.gt_profile_enable(1)
                pms, _ = timed(pearson_step, k, 1)
                lib.gt_profile_enable(0)
                gms = ctypes.c_double(0); gn = ctypes.c_uint64(0)
                lib.gt_profile_kernel_ms(b"pearson_gram", ctypes.byref(gms), ctypes.byref(gn))
                paths[pth] = {"entries_per_s": entries / (pms * 1e-3), "ms_per_step": pms,
                              "gram_ms": gms.value / max(1, gn.value), **max_err(corr)}
            except _lib.GpuToolsError as e:
                paths[pth] = {"unavailable": str(e)}
        for pth, rec in paths.items():
            if "max_rel_err_r_ge_0.01" in rec:
                rec["meets_1e-6_rel_bar"] = rec["max_rel_err_r_ge_0.01"] <= 1e-6
        if "fp32" in paths and "entries_per_s" in paths["fp32"]:
            for rec in paths.values():
                if "entries_per_s" in rec:
                    rec["x_fp32_path"] = rec["entries_per_s"] / paths["fp32"]["entries_per_s"]
        g.set_gram_path(headline)

    # end to end through the host C ABI, copies inside the timed region: with
    # ordinary pageable numpy buffers (what R's .C hands the library; gt_pmcc
    # runs the banded pipeline into them), and with page-locked buffers
    del corr, ts, pairs
    torch.cuda.empty_cache()
    e2e_steps = max(3, args.steps // 4)
    fp = lambda a: a.ctypes.data_as(ctypes.c_void_p)

    def e2e_time(hX, hp, hc, ht):
        step = lambda: _lib.check(lib.gt_pmcc(0, hX, P, hX, P, N_OBS, hp, hc, ht))
        step()
        ranks.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            step()
        return ranks.max((time.perf_counter() - t0) / e2e_steps)

    # pageable: numpy arrays with every page written before the call, as R's
    # vectors are (.C passes filled copies; np.zeros would leave them unmapped)
    nX = np.ascontiguousarray(X)
    nbufs = [np.full((P, P), 0.0, np.float32) for _ in range(3)]
    e2e_s = e2e_time(fp(nX), *(fp(b) for b in nbufs))
    del nbufs
    hX = torch.from_numpy(X).pin_memory()
    pbufs = [torch.empty((P, P), dtype=torch.float32).pin_memory() for _ in range(3)]
    e2e_pinned_s = e2e_time(vp(hX), *(vp(b) for b in pbufs))
    del pbufs, hX
    clk = clocks.stop()

    # Euclidean precision workload (rank 0; R dist layout, 5e9 entries)
    euclid = {}
    if ranks.rank == 0 and not args.skip_euclid:
        euclid = run_euclid(args, lib, g, _lib, stream, dev, headline)
    others = run_configs(lib, g, _lib, stream, dev, args.steps) if ranks.rank == 0 else {}
    refcode = run_reference_code(lib, _lib, max(3, args.steps // 4)) if ranks.rank == 0 else {}

    if ranks.rank != 0:
        return
    flops = 2.0 * N_OBS * (P * (P + 1) / 2.0)   # useful flops per Gram launch
    gram_avg_ms = gram_ms.value / max(1, gram_n.value)
    tc = headline != "fp32"
    if tc:
        # the tensor-core fraction counts the issued MMA flops: every useful
        # flop of the split encodings is 3 (bf16x3, f16x3) or 6 (bf16x6,
        # f16x6) tensor-core flops.  The timed region is a burst (steps x a
        # few ms), so the peak is the measured burst rate
        peak = peaks.get("bf16_tflops", peaks.get("bf16_tflops_sustained"))
        useful = flops / (gram_avg_ms * 1e-3) / 1e12
        products = {"bf16x3": 3, "bf16x6": 6, "f16x3": 3, "f16x6": 6}[headline]
        achieved = useful * products
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "peak_kind": f"{peaks_kind} bf16 burst",
                "flops": f"issued MMA flops: {products} split products x 2*n per unique entry",
                "useful_tflops": useful, "useful_frac": useful / peak,
                "kernel": "pearson_gram (tcgen05)", "kernel_ms": gram_avg_ms,
                "traffic": load_traffic().get(f"pearson_gram_{headline}")}
    else:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak = sms * 128 * 2 * (clk["sm_max_mhz"] or 2070.0) * 1e6 / 1e12
        achieved = flops / (gram_avg_ms * 1e-3) / 1e12
        roof = {"bound": "fp32-simt", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "peak_kind": "nominal FP32 FMA rate",
                "kernel": "pearson_gram (CUDA cores)", "kernel_ms": gram_avg_ms,
                "traffic": load_traffic().get("pearson_gram_fp32")}
    threads = oracle.threads()
    line = {
        "metric": METRIC, "value": value, "unit": "entries/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": headline,
        "data": "synthetic: seeded lognormal(5,1) + U[0,1e3] column offsets",
        "config": {"workload": f"gpuCor pearson cor(x), {N_OBS} obs x {N_VARS} vars, use=everything",
                   "n_obs": N_OBS, "n_vars": N_VARS, "entries_per_step": entries,
                   "outputs": "coefficients, ts, pairs: float32 20000x20000 each",
                   "l2": "input 328 MB and outputs 4.8 GB exceed L2 (129 MB); no flush",
                   "gram_path": headline, "parallelism": "replicas" if ranks.world > 1 else "single"},
        "e2e": {"value": ranks.world * entries / e2e_s, "unit": "entries/s",
                "h2d_bytes_per_step": int(P * N_OBS * 4), "d2h_bytes_per_step": int(2 * P * P * 4),
                "api": "gt_pmcc with pageable host buffers, as R's .C passes them (the Gram "
                       "runs in 16 bands of rows into device memory; each finished band's r "
                       "and t go to the caller's buffers by a device-to-host copy on a second "
                       "stream while the next bands run; host threads fill the constant pair "
                       "counts n meanwhile)",
                "ms_per_step": e2e_s * 1e3,
                "pinned": {"value": ranks.world * entries / e2e_pinned_s,
                           "ms_per_step": e2e_pinned_s * 1e3}},
        "gpu_launches": int(launches),
        "roofline": roof,
        "precision": {**head_err, "path": headline,
                      "sample": f"{SAMPLE_ROWS} rows x {N_VARS} vs FP64 oracle"},
        "paths": paths,
        "euclid": euclid,
        "configs": others,
        "cpu_baseline": {"value": SAMPLE_ROWS * P / cpu_dt, "unit": "entries/s", "cores": threads,
                         "kind": "port",
                         "sample": f"FP64 oracle, {SAMPLE_ROWS} rows x {N_VARS} vars x {N_OBS} obs",
                         "reference_host_loops": refcode.get("host_loops")},
        "reference_gpu_path": refcode.get("gpu_path"),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_euclid(args, lib, g, _lib, stream, dev, headline):
    import torch
    import oracle
    pts = make_euclid_data()
    dP = torch.from_numpy(pts).to(dev)
    n = E_POINTS
    m = n * (n - 1) // 2
    out = torch.empty(m, dtype=torch.float32, device=dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.check(lib.gt_distances_device(ctypes.c_void_p(dP.data_ptr()), n, E_DIM,
                                           ctypes.c_void_p(out.data_ptr()), 1, 0,
                                           ctypes.c_float(2.0), sptr))

    rng = np.random.default_rng(9)
    rows = np.sort(rng.choice(n, 16, replace=False))
    want = oracle.dist(pts, "euclidean", 2.0, b=pts[rows])  # [k, x] = d(x, rows[k])

    def check():
        o = out
        errs = []
        idx = []
        for k, r in enumerate(rows):
            x = np.arange(n)
            x = x[x != r]
            i = np.maximum(x, r); j = np.minimum(x, r)
            idx.append(n * j - j * (j + 1) // 2 + i - j - 1)
        idx = np.concatenate(idx)
        got = o[torch.from_numpy(idx).to(dev)].cpu().numpy().astype(np.float64)
        w = np.concatenate([want[k][np.arange(n) != r] for k, r in enumerate(rows)])
        zero_ok = bool(np.all(got[w == 0] == 0))
        rel = np.abs(got - w) / np.maximum(w, 1e-30)
        nz = w > 0
        return float(rel[nz].max()), zero_ok, int((w == 0).sum())

    res = {"workload": f"gpuDist euclidean, {n} points x {E_DIM} dims, {E_CLUSTERS} clusters "
                       f"(sd {E_SD}), {int(E_DUP*100)}% exact duplicates, R dist layout",
           "entries_per_step": m}
    # the bf16 settings evaluate distances as bf16x6
    peaks, peaks_kind = load_peaks()
    for pth in ("bf16x6", "f16x3", "fp32") if headline != "fp32" else ("fp32",):
        g.set_gram_path(pth)
        k = max(3, args.steps // 4)
        for _ in range(1):
            step()
        torch.cuda.synchronize()
        lib.gt_profile_reset()
        lib.gt_profile_enable(1)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        lib.gt_profile_enable(0)
        ms = e0.elapsed_time(e1) / k
        rel, zero_ok, nzero = check()
        res[pth] = {"entries_per_s": m / (ms * 1e-3), "ms_per_step": ms, "max_rel_err": rel,
                    "duplicates_exact_zero": zero_ok, "zero_pairs_in_sample": nzero}
        kms = ctypes.c_double(0); kn = ctypes.c_uint64(0)
        lib.gt_profile_kernel_ms(b"euclid_gram", ctypes.byref(kms), ctypes.byref(kn))
        if kn.value and pth != "fp32":
            kernel_ms = kms.value / kn.value
            algo = m * 4.0 + n * E_DIM * 4.0  # dist entries written + points read once
            achieved = algo / (kernel_ms * 1e-3) / 1e9
            res[pth]["roofline"] = {
                "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_kind": f"{peaks_kind} copy bandwidth",
                "kernel": "euclid_gram (tcgen05)", "kernel_ms": kernel_ms,
                "traffic": load_traffic().get(f"euclid_gram_{pth}")}
    g.set_gram_path(headline)
    del out
    torch.cuda.empty_cache()
    return res


def run_case(args):
    """One workload at a chosen size, for profiler captures and size sweeps:
    prints the per-kernel CUDA-event times of the library's main kernels."""
    import torch
    import gputools_gb300 as g
    from gputools_gb300 import _lib
    lib = g.load()
    g.set_gram_path(args.path)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    rng = np.random.default_rng(5)
    n, p = args.n, args.p
    if args.case == "pearson":
        z = rng.standard_normal((p, n), dtype=np.float32)
        X = np.exp(z + np.float32(5.0), dtype=np.float32) + rng.uniform(0, 1e3, (p, 1)).astype(np.float32)
        if args.nan_frac > 0:
            X[rng.random(X.shape) < args.nan_frac] = np.nan
        dX = torch.from_numpy(X).to(dev)
        outs = [torch.empty((p, p), dtype=torch.float32, device=dev) for _ in range(3)]
        fn = lambda: _lib.check(lib.gt_pmcc_device(args.use, vp(dX), p, vp(dX), p, n, vp(outs[0]),
                                                   vp(outs[1]), vp(outs[2]), sptr))
        names = ("pearson_prologue", "pearson_gram", "pearson_pairwise")
    elif args.case == "euclid":
        centres = rng.standard_normal((1000, 128), dtype=np.float32)
        pts = centres[rng.integers(0, 1000, p)] + np.float32(1e-3) * rng.standard_normal((p, 128), dtype=np.float32)
        dP = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
        lay = 0 if args.layout == "full" else 1
        m = p * p if lay == 0 else p * (p - 1) // 2
        out = torch.empty(m, dtype=torch.float32, device=dev)
        fn = lambda: _lib.check(lib.gt_distances_device(vp(dP), p, 128, vp(out), lay, 0,
                                                        ctypes.c_float(2.0), sptr))
        names = ("euclid_prologue", "euclid_gram", "dist")
    elif args.case == "kendall":
        X = rng.integers(0, 10, (p, n)).astype(np.float32)
        dX = torch.from_numpy(X).to(dev)
        out = torch.empty((p, p), dtype=torch.float64, device=dev)
        fn = lambda: _lib.check(lib.gt_kendall_device(vp(dX), p, vp(dX), p, n, vp(out), sptr))
        names = ("kendall_count",)
    elif args.case == "dist":
        # p points x n dims; binary on Bernoulli(0.3) 0/1 data, the others N(0,1)
        methods = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")
        mi_ = methods.index(args.metric)
        pts = ((rng.random((p, n)) < 0.3).astype(np.float32) if args.metric == "binary"
               else rng.standard_normal((p, n), dtype=np.float32))
        dP = torch.from_numpy(pts).to(dev)
        lay = 0 if args.layout == "full" else 1
        out = torch.empty(p * p if lay == 0 else p * (p - 1) // 2, dtype=torch.float32, device=dev)
        fn = lambda: _lib.check(lib.gt_distances_device(vp(dP), p, n, vp(out), lay, mi_,
                                                        ctypes.c_float(3.0), sptr))
        names = ("dist", "euclid_gram")
    elif args.case == "mi":
        # p variables x n samples sharing a common component (cor(x)-style)
        X = (rng.standard_normal((1, n)) + 0.7 * rng.standard_normal((p, n))).astype(np.float32)
        dX = torch.from_numpy(X).to(dev)
        out = torch.empty((p, p), dtype=torch.float32, device=dev)
        fn = lambda: _lib.check(lib.gt_mutual_info_device(args.bins, args.order, n, vp(dX), p,
                                                          vp(dX), p, vp(out), sptr))
        names = ("mi_prologue", "mi_gram")
    elif args.case == "batch":
        # --count cor(x) problems drawn like the batch configuration
        # (variables log-uniform in [16, 4096], observations in [50, 2000])
        gen = torch.Generator(device=dev)
        gen.manual_seed(17)
        ps = np.exp(rng.uniform(np.log(16), np.log(4096), args.count)).astype(int)
        ns = np.exp(rng.uniform(np.log(50), np.log(2000), args.count)).astype(int)
        xs = [torch.randn((int(a), int(b)), generator=gen, device=dev, dtype=torch.float32)
              for a, b in zip(ps, ns)]
        plan = g.BatchPlan(xs, "pearson", autotune=args.tune, graph=False)
        fn = lambda: plan.launch(stream)
        names = ("batch_pearson",)
    elif args.case == "cor_backward":
        # gpuCorBackward: p variables x n observations N(0,1), a symmetric p x p upstream
        dX = torch.from_numpy(rng.standard_normal((p, n), dtype=np.float32)).to(dev)
        G = torch.from_numpy(rng.standard_normal((p, p), dtype=np.float32)).to(dev)
        G = ((G + G.T) * 0.5).contiguous()
        out = torch.empty_like(dX)
        fn = lambda: _lib.check(lib.gt_cor_backward_device(vp(dX), p, n, vp(G), vp(out), sptr))
        names = ("cor_backward",)
    elif args.case == "mds":
        # MDS stress and gradient: p points x n dims N(0,1), targets uniform in [0, 8)
        dX = torch.from_numpy(rng.standard_normal((p, n), dtype=np.float32)).to(dev)
        delta = torch.from_numpy(rng.random(p * (p - 1) // 2, dtype=np.float32) * 8).to(dev)
        out = torch.empty_like(dX)
        loss = torch.zeros(1, dtype=torch.float64, device=dev)
        fn = lambda: _lib.check(lib.gt_mds_stress_device(vp(dX), p, n, vp(delta), vp(out),
                                                         vp(loss), sptr))
        names = ("mds_stress",)
    elif args.case == "hclust":
        # p points x n dims around 8 centres; each step clusters a fresh copy
        # of their euclidean distance matrix (the copy is inside the step)
        centres = rng.standard_normal((8, n)) * 4
        pts = (centres[rng.integers(0, 8, p)] + rng.standard_normal((p, n))).astype(np.float32)
        full = g.distances_device(torch.from_numpy(pts).to(dev), "euclidean").view(p, p)
        work = torch.empty_like(full)

        def fn():
            work.copy_(full)
            g.hclust_device(work, args.method, stream)
        names = ("hclust",)
    else:
        raise SystemExit(f"unknown case {args.case}")
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    lib.gt_profile_reset()
    lib.gt_profile_enable(1)
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    lib.gt_profile_enable(0)
    res = {"case": args.case, "p": p, "n": n, "path": args.path, "layout": args.layout,
           "use": args.use, "nan_frac": args.nan_frac,
           "ms_per_step": e0.elapsed_time(e1) / args.steps,
           "bk": os.environ.get("GT_TC_BK", "32"), "chunk": os.environ.get("GT_TC_CHUNK", "256")}
    for nm in names:
        ms = ctypes.c_double(); c = ctypes.c_uint64()
        lib.gt_profile_kernel_ms(nm.encode(), ctypes.byref(ms), ctypes.byref(c))
        if c.value:
            res[nm + "_ms"] = ms.value / c.value
    print(json.dumps(res), flush=True)


def run_configs(lib, g, _lib, stream, dev, steps):
    """The other configurations at their stated sizes: all six gpuDist methods
    on 4000 x 100, gpuCor kendall (500 obs x 1000 integer variables, bit-exact
    spot check) and pearson (500 x 1000), gpuDist euclidean 2000 x 64 through
    the host C ABI, the adjoints (gpuCorBackward 1024 x 4096 with a
    symmetric 4096 x 4096 upstream; MDS stress on 8192 x 32), gpuMi
    (2000 variables x 1000 samples, 10 bins, order 3) and gpuHclust (10000
    points, average linkage)."""
    import torch
    import oracle
    sptr = ctypes.c_void_p(stream.cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    rng = np.random.default_rng(21)
    out = {}

    def ev_time(fn, k):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    k = max(3, steps // 2)
    # six metrics, 4000 x 100
    base = torch.from_numpy(rng.standard_normal((4000, 100), dtype=np.float32)).to(dev)
    bern = torch.from_numpy((rng.random((4000, 100)) < 0.3).astype(np.float32)).to(dev)
    dout = torch.empty(4000 * 4000, dtype=torch.float32, device=dev)
    methods = {}
    for mi, m in enumerate(("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")):
        pts = bern if m == "binary" else base
        pw = 3.0 if m == "minkowski" else 2.0
        fn = lambda: _lib.check(lib.gt_distances_device(vp(pts), 4000, 100, vp(dout), 0, mi,
                                                        ctypes.c_float(pw), sptr))
        ms = ev_time(fn, k)
        methods[m] = {"ms": ms, "entries_per_s": 4000 * 4000 / (ms * 1e-3)}
    out["dist_4000x100"] = methods
    # kendall 500 obs x 1000 variables, integers 0..9
    Xk = rng.integers(0, 10, (1000, 500)).astype(np.float32)
    dXk = torch.from_numpy(Xk).to(dev)
    tau = torch.empty((1000, 1000), dtype=torch.float64, device=dev)
    lib.gt_profile_reset(); lib.gt_profile_enable(1)
    ms = ev_time(lambda: _lib.check(lib.gt_kendall_device(vp(dXk), 1000, vp(dXk), 1000, 500,
                                                          vp(tau), sptr)), k)
    lib.gt_profile_enable(0)
    cms = ctypes.c_double(); cn = ctypes.c_uint64()
    lib.gt_profile_kernel_ms(b"kendall_count", ctypes.byref(cms), ctypes.byref(cn))
    cols = rng.choice(1000, 6, replace=False); rows = rng.choice(1000, 6, replace=False)
    want, *_ = oracle.kendall(Xk[cols], Xk[rows], same=False)
    got = tau.cpu().numpy()[np.ix_(rows, cols)]
    for a in range(6):
        for b_ in range(6):
            if rows[a] == cols[b_]:
                want[a, b_] = 1.0
    words = (500 // 2) * ((500 + 31) // 32)
    pairs_tiles = 16 * 17 // 2 * 64 * 64          # 64 x 64 tiles on the upper triangle
    count_ms = cms.value / max(1, cn.value)
    out["kendall_500x1000"] = {
        "ms": ms, "entries_per_s": 1e6 / (ms * 1e-3), "count_kernel_ms": count_ms,
        "word_pairs_per_s": pairs_tiles * words / (count_ms * 1e-3),
        "bit_exact_sample": bool(np.array_equal(got, want))}
    # pearson 500 x 1000 and euclid 2000 x 64 end to end through the host ABI
    Xp = rng.standard_normal((1000, 500)).astype(np.float32)
    hc = np.empty((1000, 1000), np.float32); ht = np.empty_like(hc); hp = np.empty_like(hc)
    fp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _lib.check(lib.gt_pmcc(0, fp(Xp), 1000, fp(Xp), 1000, 500, fp(hp), fp(hc), fp(ht)))  # warm-up
    t0 = time.perf_counter()
    for _ in range(k):
        _lib.check(lib.gt_pmcc(0, fp(Xp), 1000, fp(Xp), 1000, 500, fp(hp), fp(hc), fp(ht)))
    out["pearson_500x1000_e2e"] = {"ms": (time.perf_counter() - t0) / k * 1e3}
    pts = rng.standard_normal((2000, 64)).astype(np.float32)
    hd = np.empty((2000, 2000), np.float32)
    _lib.check(lib.gt_distances(fp(pts), 2000, 64, fp(hd), 0, ctypes.c_float(2.0)))  # warm-up
    t0 = time.perf_counter()
    for _ in range(k):
        _lib.check(lib.gt_distances(fp(pts), 2000, 64, fp(hd), 0, ctypes.c_float(2.0)))
    out["euclid_2000x64_e2e"] = {"ms": (time.perf_counter() - t0) / k * 1e3}
    # adjoints
    Xb = torch.from_numpy(rng.standard_normal((4096, 1024), dtype=np.float32)).to(dev)
    Gb = torch.from_numpy(rng.standard_normal((4096, 4096), dtype=np.float32)).to(dev)
    Gb = (Gb + Gb.T) * 0.5
    dXb = torch.empty_like(Xb)
    ms = ev_time(lambda: _lib.check(lib.gt_cor_backward_device(vp(Xb), 4096, 1024, vp(Gb),
                                                               vp(dXb), sptr)), k)
    peaks, peaks_kind = load_peaks()
    useful = 2 * 4096 * 4096 * 1024 / (ms * 1e-3) / 1e12
    prods = {"f16x3": 3, "f16x6": 3, "bf16x3": 3, "bf16x6": 6}.get(g.get_gram_path(), 1)
    out["cor_backward_1024x4096"] = {
        "ms": ms, "useful_tflops": useful,
        "roofline": {"bound": "tensor", "achieved": useful * prods, "peak": peaks["bf16_tflops"],
                     "unit": "TFLOP/s", "frac": useful * prods / peaks["bf16_tflops"],
                     "peak_kind": f"{peaks_kind} bf16 burst",
                     "flops": f"whole call: the W = (G + G^T) Z GEMM's {prods} split products "
                              "x 2 p^2 n, over the call's time (prologue, operand splits and "
                              "the rank-1 finish included)"}}
    Xm = torch.from_numpy(rng.standard_normal((8192, 32), dtype=np.float32)).to(dev)
    delta = torch.from_numpy(rng.random(8192 * 8191 // 2, dtype=np.float32) * 8).to(dev)
    gm = torch.empty_like(Xm)
    loss = torch.zeros(1, dtype=torch.float64, device=dev)
    ms = ev_time(lambda: _lib.check(lib.gt_mds_stress_device(vp(Xm), 8192, 32, vp(delta), vp(gm),
                                                             vp(loss), sptr)), k)
    # fused CUDA-core pass: per ordered pair the distance (3 flop per
    # dimension), the weight and the accumulation (2 flop per dimension)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sms * 128 * 2 * 2070e6 / 1e12
    mds_tf = 8192 * 8191 * (5 * 32 + 8) / (ms * 1e-3) / 1e12
    out["mds_stress_8192x32"] = {
        "ms": ms, "pairs_per_s": 8192 * 8191 / (ms * 1e-3),
        "roofline": {"bound": "fp32-simt", "achieved": mds_tf, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": mds_tf / fp32_peak,
                     "peak_kind": "nominal FP32 FMA rate at 2070 MHz",
                     "flops": "5 flop per dimension + 8 per ordered pair"}}
    # above 64 dimensions: GEMMs plus the rank-1 correction on the tensor cores
    Xw = torch.from_numpy(rng.standard_normal((8192, 256), dtype=np.float32)).to(dev)
    gw = torch.empty_like(Xw)
    ms = ev_time(lambda: _lib.check(lib.gt_mds_stress_device(vp(Xw), 8192, 256, vp(delta),
                                                             vp(gw), vp(loss), sptr)), k)
    out["mds_stress_8192x256"] = {"ms": ms, "pairs_per_s": 8192 * 8191 / (ms * 1e-3),
                                  "path": "tcgen05: distances, W planes, W X"}
    del Xw, gw
    del Xb, Gb, dXb, Xm, delta, gm
    # gpuMi: 2000 variables x 1000 samples, 10 bins, cubic B-splines (order 3),
    # the symmetric all-pairs matrix; tensor cores and the CUDA-core path, and
    # a spot check of 4 rows against the FP64 oracle
    Xi = (rng.standard_normal((1, 1000)) + 0.7 * rng.standard_normal((2000, 1000))).astype(np.float32)
    dXi = torch.from_numpy(Xi).to(dev)
    mi = torch.empty((2000, 2000), dtype=torch.float32, device=dev)
    run_mi = lambda: _lib.check(lib.gt_mutual_info_device(10, 3, 1000, vp(dXi), 2000, vp(dXi), 2000,
                                                          vp(mi), sptr))
    ms = ev_time(run_mi, k)
    rows = np.array([0, 999, 1500, 1999])
    want, _, _ = oracle.bspline_mi(Xi, Xi[rows], bins=10, order=3)
    err = float(np.max(np.abs(mi.cpu().numpy()[rows].astype(np.float64) - want)))
    old_path = g.get_gram_path()
    g.set_gram_path("fp32")
    ms_cc = ev_time(run_mi, max(1, k // 3))
    g.set_gram_path(old_path)
    out["mi_2000x1000_b10_o3"] = {"ms": ms, "pairs_per_s": 2000 * 2000 / (ms * 1e-3),
                                  "cuda_core_ms": ms_cc, "max_abs_err_sample": err}
    del dXi, mi
    torch.cuda.empty_cache()
    out["hclust"] = run_hclust(g, dev)
    out["batch"] = run_batches(g, stream, dev, k)
    return out


def run_reference_code(lib, _lib, k):
    """The reference's own code, where it is built on this host from the
    staged reference sources (oracle/build_ref.sh, oracle/build_ref_gpu.sh):
    its host loops single-threaded (distance_host, src/distance.cpp:174-207;
    permHostKendall, src/correlation.cpp:506-516) and its GPU path
    (pmcc, src/correlation.cpp:66-161, and distance(), src/distance.cpp:259-316,
    with the kernels of inst/cuda, through the same host-buffer calls) beside
    this library's host entry on the same inputs: gpuCor's 500 x 1000 and
    gpuDist's 2000 x 64 configurations."""
    import oracle
    out = {}
    rng = np.random.default_rng(31)
    fp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    pts = rng.standard_normal((2000, 64)).astype(np.float32)
    Xp = rng.standard_normal((1000, 500)).astype(np.float32)
    if oracle.ref_available():
        t0 = time.perf_counter()
        oracle.ref_distance_host(pts, "euclidean")
        dt = time.perf_counter() - t0
        Xk = rng.integers(0, 10, (1000, 500)).astype(np.float32)
        t0 = time.perf_counter()
        oracle.ref_host_kendall(Xk[:4], Xk)
        dk = time.perf_counter() - t0
        out["host_loops"] = {
            "cores": 1, "compiled": "g++ -O3 from the reference's src/*.cpp",
            "distance_host_euclidean_2000x64": {"s": dt, "entries_per_s": 2000 * 2000 / dt},
            "permHostKendall_500obs": {"sample": "4 x 1000 variable pairs", "s": dk,
                                       "entries_per_s": 4000 / dk}}
    if oracle.ref_gpu_available():
        rec = {"kernels": "the reference's inst/cuda kernels, nvcc --use_fast_math for sm_103a, "
                          "launched by name; its host code allocates, copies and frees per call"}
        Xb = Xp.copy()  # R's .C passes two copies of x
        hc = np.empty((1000, 1000), np.float32); ht = np.empty_like(hc); hp = np.empty_like(hc)
        oracle.ref_gpu_pmcc(Xp, Xb)
        t0 = time.perf_counter()
        for _ in range(k):
            rc_, _, _ = oracle.ref_gpu_pmcc(Xp, Xb)
        ref_ms = (time.perf_counter() - t0) / k * 1e3
        _lib.check(lib.gt_pmcc(0, fp(Xp), 1000, fp(Xb), 1000, 500, fp(hp), fp(hc), fp(ht)))
        t0 = time.perf_counter()
        for _ in range(k):
            _lib.check(lib.gt_pmcc(0, fp(Xp), 1000, fp(Xb), 1000, 500, fp(hp), fp(hc), fp(ht)))
        ours_ms = (time.perf_counter() - t0) / k * 1e3
        rec["pearson_500x1000"] = {"reference_ms": ref_ms, "ours_ms": ours_ms,
                                   "speedup": ref_ms / ours_ms,
                                   "max_abs_diff_r": float(np.abs(rc_ - hc).max())}
        hd = np.empty((2000, 2000), np.float32)
        oracle.ref_gpu_distance(pts, "euclidean")
        t0 = time.perf_counter()
        for _ in range(k):
            rd = oracle.ref_gpu_distance(pts, "euclidean")
        ref_ms = (time.perf_counter() - t0) / k * 1e3
        _lib.check(lib.gt_distances(fp(pts), 2000, 64, fp(hd), 0, ctypes.c_float(2.0)))
        t0 = time.perf_counter()
        for _ in range(k):
            _lib.check(lib.gt_distances(fp(pts), 2000, 64, fp(hd), 0, ctypes.c_float(2.0)))
        ours_ms = (time.perf_counter() - t0) / k * 1e3
        rec["euclid_2000x64"] = {"reference_ms": ref_ms, "ours_ms": ours_ms,
                                 "speedup": ref_ms / ours_ms,
                                 "max_rel_diff": float(np.max(np.abs(rd - hd) / np.maximum(hd, 1e-3)))}
        out["gpu_path"] = rec
    return out


def run_hclust(g, dev):
    """gpuHclust, average linkage, on the euclidean distances of 10000 points
    in 16 dimensions drawn around 8 centres: the merge loop alone (a fresh
    copy of the device matrix per call; the call returns merges, order and
    heights on the host), and gpuDistClust end to end from host points.  The
    oracle runs on the first 1000 points (its loop rescans every row each
    step, O(n^3)) for the CPU rate and an exact comparison of the merges."""
    import torch
    import oracle
    rng = np.random.default_rng(31)
    n, d = 10000, 16
    centres = rng.standard_normal((8, d)) * 4
    pts = (centres[rng.integers(0, 8, n)] + rng.standard_normal((n, d))).astype(np.float32)
    dp = torch.from_numpy(pts).to(dev)
    full = g.distances_device(dp, "euclidean").view(n, n)
    work = torch.empty_like(full)
    times = []
    for rep in range(3):
        work.copy_(full)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.hclust_device(work, "average")
        times.append(time.perf_counter() - t0)
    ms = min(times[1:]) * 1e3
    del work, full, dp
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    g.gpuDistClust(pts, "euclidean", "average")
    e2e_ms = (time.perf_counter() - t0) * 1e3
    m = 1000
    sub = g.gpuDist(pts[:m])
    dm = sub.to_matrix().astype(np.float32)
    t0 = time.perf_counter()
    s_, p_, h_ = oracle.hclust(dm, "average")
    cpu_ms = (time.perf_counter() - t0) * 1e3
    om, oo = oracle.format_clustering(s_, p_)
    res = g.gpuHclust(sub, "average")
    exact = bool(np.array_equal(res.merge, om) and np.array_equal(res.order, oo)
                 and np.array_equal(res.height.view(np.int32), h_.view(np.int32)))
    return {"average_10000x16": {"ms": ms, "us_per_merge": ms * 1e3 / (n - 1),
                                 "gpuDistClust_e2e_ms": e2e_ms},
            "oracle_cpu_1000_ms": cpu_ms, "oracle_cpu_threads": oracle.threads(),
            "exact_vs_oracle_1000": exact}


def run_batches(g, stream, dev, k):
    """2000 independent Pearson problems (variables log-uniform in [16, 4096],
    observations log-uniform in [50, 2000], N(0,1)) and 500 Kendall problems
    (200 observations, log-uniform [8, 512] integer variables 0..19), each batch
    one plan replayed from a CUDA graph."""
    import torch
    gen = torch.Generator(device=dev)
    gen.manual_seed(17)
    rng = np.random.default_rng(17)
    res = {}
    ps = np.exp(rng.uniform(np.log(16), np.log(4096), 2000)).astype(int)
    ns = np.exp(rng.uniform(np.log(50), np.log(2000), 2000)).astype(int)
    xs = [torch.randn((int(p), int(n)), generator=gen, device=dev, dtype=torch.float32)
          for p, n in zip(ps, ns)]
    entries = float(np.sum(ps.astype(np.float64) ** 2))
    useful = float(np.sum(2.0 * ps.astype(np.float64) ** 2 * ns))
    # batches run the f16x3 split (the plan takes the Gram path at creation)
    old_path = g.get_gram_path()
    g.set_gram_path("f16x3")
    t0 = time.perf_counter()
    try:
        plan = g.BatchPlan(xs, "pearson", autotune=True)
    finally:
        g.set_gram_path(old_path)
    build_s = time.perf_counter() - t0
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    plan.launch(stream)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k):
        plan.launch(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / k
    peaks, peaks_kind = load_peaks()
    # algorithmic bytes: r, t and pairs written (12 bytes per entry), the
    # inputs read, the two f16 operand planes written and read once
    kpad = (ns.astype(np.float64) + 63) // 64 * 64
    pf = ps.astype(np.float64)
    nbytes = 12 * entries + 4 * float(np.sum(pf * ns)) + 8 * float(np.sum(pf * kpad))
    out_gbs = nbytes / (ms * 1e-3) / 1e9
    res["pearson_2000"] = {"ms": ms, "entries": entries, "entries_per_s": entries / (ms * 1e-3),
                           "useful_tflops": useful / (ms * 1e-3) / 1e12, "plan": plan.describe(),
                           "plan_build_s": build_s, "launches_per_step": "1 graph",
                           "outputs": "p x p views of pitched storage (rows a multiple of 8 "
                                      "floats apart)",
                           "roofline": {"bound": "hbm", "achieved": out_gbs,
                                        "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                        "frac": out_gbs / peaks["hbm_gbs"],
                                        "peak_kind": f"{peaks_kind} copy bandwidth",
                                        "bytes": "outputs (12 B per entry), inputs, operand "
                                                 "planes written and read once",
                                        "algorithmic_bytes": nbytes}}
    plan.close()
    del xs
    torch.cuda.empty_cache()
    kp = np.exp(rng.uniform(np.log(8), np.log(512), 500)).astype(int)
    ks = [torch.from_numpy(rng.integers(0, 20, (int(p), 200)).astype(np.float32)).to(dev)
          for p in kp]
    plan = g.BatchPlan(ks, "kendall")
    plan.launch(stream)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k):
        plan.launch(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / k
    kent = float(np.sum(kp.astype(np.float64) ** 2))
    res["kendall_500"] = {"ms": ms, "entries": kent, "entries_per_s": kent / (ms * 1e-3),
                          "plan": plan.describe()}
    plan.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--skip-euclid", action="store_true")
    ap.add_argument("--count", type=int, default=300, help="--case batch: problems")
    ap.add_argument("--tune", action="store_true", help="--case batch: autotune the plan")
    ap.add_argument("--case", choices=("pearson", "euclid", "kendall", "dist", "mi", "hclust",
                                       "batch", "cor_backward", "mds"),
                    help="run one workload at the given size instead of the benchmark")
    ap.add_argument("--p", type=int, default=4096, help="--case: variables / points")
    ap.add_argument("--n", type=int, default=4096, help="--case: observations")
    ap.add_argument("--path", default="bf16x3", help="--case: gram path")
    ap.add_argument("--layout", default="dist", help="--case euclid: full or dist")
    ap.add_argument("--metric", default="manhattan", help="--case dist: distance method")
    ap.add_argument("--bins", type=int, default=10, help="--case mi: bins")
    ap.add_argument("--order", type=int, default=3, help="--case mi: spline order")
    ap.add_argument("--method", default="average", help="--case hclust: linkage")
    ap.add_argument("--use", type=int, default=0,
                    help="--case pearson: 0 everything, 1 pairwise.complete.obs")
    ap.add_argument("--nan-frac", type=float, default=0.0,
                    help="--case pearson: fraction of values set to NaN")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        # rank 0 alone times the CPU implementation; other ranks have no work
        world, rank, _ = dist_env()
        if rank == 0:
            run_reference(args, type("R", (), {"rank": 0})())
        return
    ranks = Ranks()
    try:
        run_ours(args, ranks)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
