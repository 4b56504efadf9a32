"""The R package overlay (rpkg/): src/Makevars and the R gradient wrappers.

R is not installed here, so these are checked as text against the built
library, which is what R would bind them to:
  * `make -n` on rpkg/src/Makevars compiles every CUDA source of the library
    with nvcc for sm_103a, one object each;
  * every .C("name", ...) in rpkg/R/*.R names a symbol the library exports,
    with as many positional arguments as the C declaration in
    include/gputools_gb300.h has parameters;
  * the same holds for the reference's own R callers of the hot path
    (R/gpuCor.R, R/gpuHclust.R, R/gpuMi.R, R/zzz.R) when the reference tree
    is present (GPUTOOLS_REFERENCE or the benchmark's reference_path).
"""
import glob
import json
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RPKG = os.path.join(ROOT, "rpkg")
HEADER = os.path.join(ROOT, "include", "gputools_gb300.h")
NAMED = ("PACKAGE", "NAOK", "DUP", "ENCODING")


def c_calls(text):
    """(name, positional argument count) of every .C call in R source."""
    out = []
    for m in re.finditer(r'\.C\(\s*"([A-Za-z_][A-Za-z0-9_]*)"', text):
        depth, i, start, args = 1, m.end(), m.end(), []
        while depth:
            ch = text[i]
            if ch in "([{":
                depth += 1
            elif ch in ")]}":
                depth -= 1
            elif ch == "," and depth == 1:
                args.append(text[start:i])
                start = i + 1
            i += 1
        args.append(text[start:i - 1])
        pos = [a for a in args if a.strip() and not re.match(r"\s*(%s)\s*=" % "|".join(NAMED), a)]
        out.append((m.group(1), len(pos)))
    return out


def header_params():
    """Parameter count of every void-returning function in the C header."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    params = {}
    for m in re.finditer(r"\bvoid\s+([A-Za-z_]\w*)\s*\(([^)]*)\)\s*;", text):
        body = m.group(2).strip()
        params[m.group(1)] = 0 if body in ("", "void") else body.count(",") + 1
    return params


@pytest.fixture(scope="module")
def exported(lib):
    from gputools_gb300 import builder
    out = subprocess.run(["nm", "-D", "--defined-only", builder.LIB], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_makevars_compiles_every_source_for_sm103a(tmp_path):
    if not shutil.which("make"):
        pytest.skip("make not installed")
    cus = sorted(os.path.basename(p) for p in glob.glob(os.path.join(ROOT, "gputools_gb300", "csrc", "*.cu")))
    objs = [c[:-3] + ".o" for c in cus]
    mk = os.path.join(RPKG, "src", "Makevars")
    show = subprocess.run(["make", "-s", "-f", mk, f"GT_ROOT={ROOT}", "--eval",
                           "show-objects: ; @echo $(OBJECTS)", "show-objects"],
                          cwd=tmp_path, capture_output=True, text=True, check=True).stdout.split()
    assert show == objs
    dry = subprocess.run(["make", "-n", "-f", mk, f"GT_ROOT={ROOT}"] + objs, cwd=tmp_path,
                         capture_output=True, text=True, check=True).stdout
    lines = [l for l in dry.splitlines() if "nvcc" in l]
    assert len(lines) == len(cus)
    for cu, line in zip(cus, lines):
        assert "arch=compute_103a,code=sm_103a" in line
        assert line.rstrip().endswith(f"-c {ROOT}/gputools_gb300/csrc/{cu} -o {cu[:-3]}.o")


def test_r_wrappers_bind_exported_symbols(exported):
    params = header_params()
    calls = []
    for f in sorted(glob.glob(os.path.join(RPKG, "R", "*.R"))):
        calls += c_calls(open(f).read())
    assert {c for c, _ in calls} == {"RgpuCorBackward", "RgpuDistBackward", "RgpuMdsStress"}
    for name, nargs in calls:
        assert name in exported, name
        assert params[name] == nargs, (name, params[name], nargs)
    ns = open(os.path.join(RPKG, "NAMESPACE.add")).read()
    for fn in ("gpuCorBackward", "gpuDistBackward", "gpuMdsStress"):
        assert fn in ns
        assert any(re.search(rf"^{fn}\s*<-\s*function", open(f).read(), re.M)
                   for f in glob.glob(os.path.join(RPKG, "R", "*.R")))


def _reference_root():
    env = os.environ.get("GPUTOOLS_REFERENCE")
    if env:
        return env
    try:
        return json.load(open(os.path.join(ROOT, "BASELINE.json"))).get("reference_path")
    except (OSError, ValueError):
        return None


def test_reference_r_callers_bind_exported_symbols(exported):
    ref = _reference_root()
    if not ref or not os.path.isdir(os.path.join(ref, "R")):
        pytest.skip("reference tree not present")
    params = header_params()
    seen = set()
    for name in ("gpuCor.R", "gpuHclust.R", "gpuMi.R", "zzz.R"):
        for sym, nargs in c_calls(open(os.path.join(ref, "R", name)).read()):
            seen.add(sym)
            assert sym in exported, (name, sym)
            assert params[sym] == nargs, (name, sym, params[sym], nargs)
    assert {"rpmcc", "RgpuKendall", "Rdistances", "rBSplineMutualInfo", "Rhcluster",
            "Rdistclust", "rtestT", "cuCompile"} <= seen
