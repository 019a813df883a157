"""bench.py's compute bounds of the cull kernel (no GPU): the warp-instruction issue and
FP32 lane-operation figures from the committed ncu counts (the warm kernel reading the box
cache and the cold fused one), scaled by object-views."""
import json

import pytest

import bench
from conftest import ROOT

CAPTURES = json.loads((ROOT / "profiles" / "cull_stress_traffic.json").read_text())


class _Workload:
    def __init__(self, n, v):
        self.n, self.v = n, v

    def object_views(self):
        return self.n * self.v


@pytest.mark.parametrize("kernel", sorted(CAPTURES))
def test_pipe_bounds_from_the_committed_capture(kernel):
    d = CAPTURES[kernel]
    wl = _Workload(d["objects"], d["views"])  # the captured case itself: scale 1
    secs = d["sm_cycles_elapsed"] / 2.0e9  # its duration at 2 GHz
    issue, fp32 = bench.pipe_bounds(wl, secs * 1e3, 2000.0, 152, kernel)
    # one warp-instruction per scheduler per cycle: the capture's own issue fraction
    assert abs(issue["frac"] - d["warp_instructions_per_launch"] / (d["sm_cycles_elapsed"] * 4 * 152)) < 1e-9
    assert 30 < issue["thread_instructions_per_object_view"] < 120
    # the plane FMAs at least: six planes (18) in the fused kernel, five (15) in the cached one,
    # which leaves out the far plane of the stress views (their scene bound clears it)
    planes = 15 if kernel == "warm" else 18
    assert 0 < fp32["frac"] < 1 and fp32["ops_per_object_view"] > planes
    # scaled to the 16M-object workload: same per-object-view figures
    issue16, fp16 = bench.pipe_bounds(_Workload(16_000_000, 8), 1.0, 2070.0, 152, kernel)
    assert abs(issue16["thread_instructions_per_object_view"] - issue["thread_instructions_per_object_view"]) < 0.01
    assert abs(fp16["ops_per_object_view"] - fp32["ops_per_object_view"]) < 0.01
    assert bench.pipe_bounds(wl, 0.0, 2000.0, 152, kernel) == (None, None)
