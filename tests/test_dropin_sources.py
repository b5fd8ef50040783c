"""The reference's own front-end sources compile UNCHANGED against this
library: its CLI (tools/gpu_pfflop.cu) and its pybind11 module
(python/pps_native.cpp) include gpu_cfr.h, postflop_cfr.h and range.h, so
with include/pps on the include path and libpps_gb.so in place of the
reference's cuda/gpu_cfr.cu + src/*.cpp they must build, link (every
symbol they call resolved by libpps_gb.so) and run.

CPU tests. They read the reference's sources where they are mounted
(PPS_REFERENCE, else a `reference` checkout beside this repository) and
skip elsewhere; the builds go to a temporary directory. Without a GPU the
run stops where the library first needs the device: the CLI's argument
errors and the binding's input errors come out as the reference's own
(exit status 2, RuntimeError), and the library's CUDA error reaches
Python as a RuntimeError instead of ending the process (the reference's
engine calls exit(1) there, cuda/gpu_cfr.cu:43-51). The library calls the
binding makes are the C++ class that the CLI built here
(pps/gpu_pfflop, the same class) drives on the GPU in
tests/test_gpu_api.py.
"""
import os
import re
import shutil
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("PPS_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
LIBDIR = os.path.join(REPO, "cuda-poker-solver_gb300", "pps")
INCLUDE = os.path.join(REPO, "include", "pps")

CLI_SRC = os.path.join(REF, "tools", "gpu_pfflop.cu")
PYBIND_SRC = os.path.join(REF, "python", "pps_native.cpp")

pytestmark = pytest.mark.skipif(
    not (os.path.exists(CLI_SRC) and os.path.exists(PYBIND_SRC)),
    reason="the reference's sources are not mounted (set PPS_REFERENCE)")


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not found")


def test_reference_cli_source_builds_against_this_library(tmp_path):
    exe = str(tmp_path / "gpu_pfflop_ref")
    r = subprocess.run([_nvcc(), "-std=c++17", "-O2", "-I", INCLUDE, CLI_SRC, "-L", LIBDIR,
                        "-lpps_gb", "-Xlinker", "-rpath", "-Xlinker", LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # The reference's usage error (tools/gpu_pfflop.cu: exit status 2).
    u = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert u.returncode == 2
    assert "usage: gpu_pfflop postflop <board>" in u.stdout + u.stderr
    # Its argument checks, before any device work.
    b = subprocess.run([exe, "postflop", "Qs9h", "TT+", "99+", "200", "3000", "0.5", "", "0"],
                       capture_output=True, text=True, timeout=60)
    assert b.returncode != 0


def _methods_bound_by(src):
    text = open(src).read()
    return sorted(set(re.findall(r'\.def(?:_static|_property_readonly)?\("([a-z_]+)"', text)))


def test_reference_pybind_source_builds_against_this_library(tmp_path):
    pybind11 = pytest.importorskip("pybind11")
    suffix = subprocess.run([sys.executable, "-c",
                             "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))"],
                            capture_output=True, text=True).stdout.strip()
    mod = str(tmp_path / ("pps_native" + suffix))
    inc = [pybind11.get_include()]
    import sysconfig
    inc.append(sysconfig.get_paths()["include"])
    cmd = ["g++", "-std=c++17", "-O1", "-shared", "-fPIC"] + sum((["-I", i] for i in inc), []) + \
        ["-I", INCLUDE, PYBIND_SRC, "-L", LIBDIR, "-lpps_gb", "-Wl,-rpath," + LIBDIR, "-o", mod]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    probe = r'''
import json, sys
sys.path.insert(0, sys.argv[1])
import pps_native as m
out = {"methods": sorted(x for x in dir(m.Solver) if not x.startswith("_"))}
def err(**kw):
    try:
        m.Solver(**kw)
        return None
    except Exception as e:
        return [type(e).__name__, str(e)]
out["bad_board"] = err(board="Qs9h", oop="TT+,AKo", ip="AQ+,KQs", pot=200, stack=500)
out["bad_range"] = err(board="Qs9h2d7c", oop="TT+,XYZ", ip="AQ+,KQs", pot=200, stack=500)
out["solve"] = err(board="Qs9h2d7c", oop="TT+,AKo", ip="AQ+,KQs", pot=200, stack=500,
                   bets="0.75,a", raises="2.5,3")
print(json.dumps(out))
'''
    p = subprocess.run([sys.executable, "-c", probe, str(tmp_path)], capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-3000:]
    import json
    out = json.loads(p.stdout.strip().splitlines()[-1])
    want = [n for n in _methods_bound_by(PYBIND_SRC) if n != "Solver"]
    assert set(want) <= set(out["methods"]), (want, out["methods"])
    assert out["bad_board"][0] == "RuntimeError" and "board" in out["bad_board"][1]
    assert out["bad_range"][0] == "RuntimeError"
    # With a GPU this spot solves; without one the library's CUDA error
    # reaches Python as an exception rather than ending the process.
    if out["solve"] is not None:
        assert out["solve"][0] == "RuntimeError" and "CUDA" in out["solve"][1]
