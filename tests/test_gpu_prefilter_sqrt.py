"""The prefilter's row norms use the hardware square root approximation on the GPU
(pipeline_gb300/csrc/dpcull_prefilter.h, sqrt_bound); its bounds stay upper bounds only if
the approximation's relative error is below the 2^-18 inflation applied after it.  Every
float input the prefilter can pass (>= 2^-120) is checked against the correctly rounded
root computed in double."""
import re
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_sqrt_approx_bound(tmp_path):
    from pipeline_gb300 import build

    exe = tmp_path / "sqrt_bound_check"
    r = subprocess.run([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                        str(ROOT / "tests" / "cpp" / "sqrt_bound_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"max_rel_err=(\S+) log2=(\S+) violations=(\d+)", r.stdout)
    assert m, r.stdout
    err, bad = float(m.group(1)), int(m.group(3))
    assert bad == 0
    assert err < 2.0 ** -21, r.stdout
