"""The Gram kernels' tile order (gputools_gb300/csrc/gram_core.cuh), checked
on the host: tests/tile_order_check.cu, built by nvcc and run without a GPU,
enumerates every tile of the full, upper and lower tile sets for many shapes
and band widths and checks that each appears exactly once."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "gputools_gb300", "csrc")


def test_tile_order_covers_each_tile_once(tmp_path):
    nvcc = shutil.which("nvcc") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                "bin", "nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "tile_order_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    os.path.join(HERE, "tile_order_check.cu"), "-lcuda"],
                   check=True, timeout=600)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stdout + res.stderr
