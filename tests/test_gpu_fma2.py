"""The cull evaluates the lo and hi plane of an axis as one fma.rn.f32x2 pair
(pipeline_gb300/csrc/cull.cu, classify_views); the prefilter's bounds are proven for, and
host-tested on, the scalar fma chain (dpcull_prefilter.h, pf::plane).  Each half of the
packed FMA must round exactly like fma.rn.f32: 2^28 seeded pairs of triples over any bit
pattern, wide-range normals, near-cancelling addends and subnormals, compared bit for bit
(both-NaN counts as equal)."""
import re
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_fma_f32x2_halves_equal_scalar_fma(tmp_path):
    from pipeline_gb300 import build

    exe = tmp_path / "fma2_check"
    r = subprocess.run([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-ftz=false",
                        str(ROOT / "tests" / "cpp" / "fma2_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"pairs=(\d+) mismatches=(\d+)", r.stdout)
    assert m, r.stdout
    assert int(m.group(1)) == 1 << 28
    assert int(m.group(2)) == 0, r.stdout
