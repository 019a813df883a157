"""The C++ host layer (dpcull::Manager, dpcull::transform::Tree) against the oracle's
stateful manager and tree, driven from a C++ program through identical operation
sequences (removals, additions, matrices changed with and without dirty marks, boxes
changed without a dirty mark, bounding boxes, several results, batched views)."""
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_manager_parity(tmp_path):
    from pipeline_gb300 import build

    build.build_all()
    exe = tmp_path / "manager_parity"
    orc = tmp_path / "cull_oracle.o"
    lib = ROOT / "pipeline_gb300" / "_lib"
    r = subprocess.run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-c",
                        str(ROOT / "oracle" / "cull_oracle.c"), "-o", str(orc)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off",
           "-I", str(ROOT / "include"), "-I", str(ROOT / "pipeline_gb300" / "cpp"), "-I", str(ROOT / "oracle"),
           str(ROOT / "tests" / "cpp" / "manager_parity.cpp"), str(orc), "-o", str(exe),
           "-L", str(lib), "-ldpcull_mgr", "-ldpcull", f"-Wl,-rpath,{lib}", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all sequences equal" in r.stdout
