"""The C ABI library loads and exports what include/gputools_gb300.h declares,
and the host-side argument handling behaves like the reference (CPU only: no
call here reaches a device)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gputools_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))


def test_header_declares_reference_symbols():
    names = declared_functions()
    for sym in ("Rdistances", "rpmcc", "RgpuKendall", "rsetDevice", "rgetDevice", "rtestT",
                "cuCompile", "unloadPackage"):
        assert sym in names


def test_library_exports_every_declared_symbol(lib):
    from gputools_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if " T " in line)
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    # the Python binding covers exactly the declared set
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_build_targets_sm_103a_only():
    from gputools_gb300 import builder
    assert builder.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_status_api_rejects_bad_arguments_without_a_device(lib):
    assert lib.gt_distances(None, -1, 3, None, 0, 2.0) == 1
    assert "negative" in lib.gt_last_error().decode()
    assert lib.gt_distances(None, 4, 3, None, 9, 2.0) == 1
    assert "unknown distance method" in lib.gt_last_error().decode()
    assert lib.gt_pmcc(7, None, 1, None, 1, 3, None, None, None) == 1
    assert lib.gt_last_error().decode() == "unknown use method"
    assert lib.gt_kendall(None, 1, None, 1, 70000, None) == 1
    assert lib.gt_set_gram_path(42) == 1
    assert lib.gt_version() == 10000


def test_rpmcc_unknown_use_reports_reference_message(lib):
    w = ctypes.c_int(5); one = ctypes.c_int(1)
    lib.rpmcc(ctypes.byref(w), None, ctypes.byref(one), None, ctypes.byref(one),
              ctypes.byref(one), None, None, None)
    assert lib.gt_last_error().decode() == "unknown use method"


def test_empty_problems_are_no_ops(lib):
    assert lib.gt_distances(None, 0, 5, None, 0, 2.0) == 0
    assert lib.gt_pmcc(0, None, 0, None, 3, 10, None, None, None) == 0
    assert lib.gt_kendall(None, 0, None, 0, 10, None) == 0


def test_pmatch_semantics():
    from gputools_gb300 import pmatch
    t = ("euclidean", "maximum", "manhattan", "canberra", "binary", "minkowski")
    assert pmatch("euclidean", t) == 0
    assert pmatch("man", t) == 2
    assert pmatch("m", t) is None          # ambiguous
    assert pmatch("", t) is None
    assert pmatch("mink", t) == 5


def test_r_api_argument_errors(lib):
    import gputools_gb300 as g
    with pytest.raises(ValueError, match="invalid distance method"):
        g.gpuDist(np.ones((3, 2)), "m")
    with pytest.raises(ValueError, match="NA/NaN/Inf"):
        g.gpuDist(np.array([[1.0, np.nan], [0.0, 1.0]]))
    with pytest.raises(ValueError, match="ambiguous correlation method"):
        g.gpuCor(np.ones((3, 2)), method="spearman")


def test_dist_object_layout():
    from gputools_gb300 import Dist
    n = 4
    m = np.arange(n * n, dtype=np.float64).reshape(n, n)
    m = m + m.T
    np.fill_diagonal(m, 0)
    cols, rows = np.triu_indices(n, 1)
    d = Dist(m[cols, rows], n, "euclidean")
    # R order: (2,1),(3,1),(4,1),(3,2),(4,2),(4,3)
    assert list(d.values) == [m[1, 0], m[2, 0], m[3, 0], m[2, 1], m[3, 1], m[3, 2]]
    np.testing.assert_array_equal(d.to_matrix(), m)


def test_problem_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the batch problem structs have the header's size
    and field offsets (a C program compiled against the header prints them)."""
    from gputools_gb300 import _lib
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "gputools_gb300.h"\n'
        "int main(void) {\n"
        '  printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gt_cor_problem),\n'
        "         offsetof(gt_cor_problem, X), offsetof(gt_cor_problem, p),\n"
        "         offsetof(gt_cor_problem, n), offsetof(gt_cor_problem, corr),\n"
        "         offsetof(gt_cor_problem, ts), offsetof(gt_cor_problem, pairs),\n"
        "         offsetof(gt_cor_problem, ld));\n"
        '  printf("%zu %zu %zu %zu %zu\\n", sizeof(gt_kendall_problem),\n'
        "         offsetof(gt_kendall_problem, X), offsetof(gt_kendall_problem, p),\n"
        "         offsetof(gt_kendall_problem, n), offsetof(gt_kendall_problem, out));\n"
        "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True,
                           check=True).stdout.split("\n")
    cor = [int(v) for v in lines[0].split()]
    ken = [int(v) for v in lines[1].split()]
    C, K = _lib.CorProblem, _lib.KendallProblem
    assert cor == [ctypes.sizeof(C)] + [getattr(C, f).offset
                                        for f in ("X", "p", "n", "corr", "ts", "pairs", "ld")]
    assert ken == [ctypes.sizeof(K)] + [getattr(K, f).offset for f in ("X", "p", "n", "out")]
