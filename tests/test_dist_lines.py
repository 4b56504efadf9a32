"""The aligned-line tiling of the dist layout (gputools_gb300/csrc/dist_lines.cuh),
checked on the host: tests/dist_lines_check.cpp builds the header with g++
and verifies, for several n and output offsets, that the permuted column
operand is a bijection, that every tile column starts each warp's 32 rows on
a 128-byte line, that the tiles enumerate each (row tile, super-block, class)
once, and (n <= 12000) that every dist entry is computed exactly once.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gputools_gb300", "csrc")


def test_dist_lines_tiling(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "dist_lines_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-o", str(exe),
                    os.path.join(HERE, "dist_lines_check.cpp")], check=True)
    sizes = ["2", "3", "31", "64", "65", "127", "129", "700", "8191", "8192", "8193",
             "12000", "100000", "379000"]
    res = subprocess.run([str(exe)] + sizes, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and res.stdout.strip() == "ok", res.stdout + res.stderr
