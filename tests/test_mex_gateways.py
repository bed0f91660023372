"""The MATLAB gateways compile against the C ABI header (a syntax and type
check with a stub mex.h: MATLAB is not installed), and every C entry point
they call is exported by the engine library's header."""
import glob
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MEX = os.path.join(ROOT, "gpumatfun_gb300", "mex")
GATEWAYS = sorted(glob.glob(os.path.join(MEX, "*.cpp")))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("src", GATEWAYS, ids=[os.path.basename(g) for g in GATEWAYS])
def test_gateway_compiles(src):
    stub = os.path.join(ROOT, "tests", "mexstub")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", stub, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_gateways_listed_in_build_script():
    script = open(os.path.join(MEX, "build_mex.m")).read()
    listed = set(re.findall(r"'(\w+)'", script))
    for g in GATEWAYS:
        assert os.path.splitext(os.path.basename(g))[0] in listed


def test_gateways_call_declared_entry_points():
    header = open(os.path.join(ROOT, "include", "gpumatfun.h")).read()
    declared = set(re.findall(r"\b(gm_\w+)\s*\(", header))
    for g in GATEWAYS + [os.path.join(MEX, "gm_mex_common.h")]:
        for name in set(re.findall(r"\b(gm_[a-z_]+)\s*\(", open(g).read())):
            if name.startswith("gm_mex_"):
                continue
            assert name in declared, (g, name)
