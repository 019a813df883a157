"""The cull's conservative prefilter (pipeline_gb300/csrc/dpcull_prefilter.h), compiled for
the host from the same source as the kernels, against the oracle's exact visibility
(dp/culling/cpu/src/ManagerImpl.cpp:263-289): wherever the prefilter decides a pair, the
decision must equal the reference's rounded result.  Families: the benchmark
distributions under cube, stereo, cascade and random perspective views; boxes centred on
the frustum planes at every scale; projective world matrices (always undecided); extreme
coordinates and clip ranges; non-finite values.  A build with a deliberately weakened
margin must disagree somewhere, which shows that the families reach the rounding
boundary."""
import ctypes
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT
from pipeline_gb300 import workloads as wl


def _build(tmp_path, name, extra=()):
    so = tmp_path / f"{name}.so"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", *extra,
           "-I", str(ROOT / "pipeline_gb300" / "csrc"), str(ROOT / "tests" / "cpp" / "prefilter_host.cpp"),
           "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(str(so))
    lib.pf_classify_soa.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 6
    lib.pf_classify_soa.restype = None
    lib.pf_classify_group_soa.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 5 + [ctypes.c_size_t, ctypes.c_void_p]
    lib.pf_classify_group_soa.restype = None
    return lib


@pytest.fixture(scope="module", params=["loose", "tight"])
def pf(request, tmp_path_factory):
    """The prefilter with the radius the fused kernel computes every launch ("loose") and
    with the one the Fill launch stores in the box cache ("tight"): every family runs
    with both."""
    extra = ["-DPF_TIGHT"] if request.param == "tight" else []
    return _build(tmp_path_factory.mktemp("pf"), "pf_" + request.param, extra)


@pytest.fixture(scope="module")
def pf_weak(tmp_path_factory):
    return _build(tmp_path_factory.mktemp("pfw"), "pfw", ["-DDPCULL_PF_TEST_DELTA=0.0f"])


def classify(lib, lower, extent, xform, mats, vp):
    n = lower.shape[1]
    out = np.empty(n, np.int8)
    args = [np.ascontiguousarray(a) for a in (lower, extent, xform, mats, np.asarray(vp, np.float32).reshape(16))]
    lib.pf_classify_soa(n, *[a.ctypes.data for a in args], out.ctypes.data)
    return out


def classify_group(lib, lower, extent, xform, mats, vps):
    """Every view of vps decided against the group margin of all of them: [views, n]."""
    n = lower.shape[1]
    vps = np.ascontiguousarray(np.asarray(vps, np.float32).reshape(-1, 16))
    out = np.empty((vps.shape[0], n), np.int8)
    args = [np.ascontiguousarray(a) for a in (lower, extent, xform, mats)]
    lib.pf_classify_group_soa(n, *[a.ctypes.data for a in args], vps.ctypes.data, vps.shape[0], out.ctypes.data)
    return out


def exact(lower, extent, xform, mats, vp):
    n = lower.shape[1]
    bits = oracle.cull_bits(lower, extent, xform, mats, vp)
    return ((bits[np.arange(n) >> 5] >> (np.arange(n) & 31).astype(np.uint32)) & 1).astype(bool)


def check(lib, scene, vps, group: int = 8):
    """Returns (pairs, decided, wrong) over all views: each view decided alone and the
    views decided in groups of `group` consecutive views against the group margin (as the
    multi-view kernels do); decided counts the grouped decisions, wrong counts both."""
    pairs = decided = wrong = 0
    vps = [np.asarray(v, np.float32).reshape(16) for v in vps]
    ex = [exact(*scene, vp) for vp in vps]
    for vp, e in zip(vps, ex):
        cls = classify(lib, *scene, vp)
        wrong += int(np.count_nonzero((cls != 2) & ((cls == 1) != e)))
    for g0 in range(0, len(vps), group):
        cls = classify_group(lib, *scene, vps[g0:g0 + group])
        for k, c in enumerate(cls):
            dec = c != 2
            wrong += int(np.count_nonzero(dec & ((c == 1) != ex[g0 + k])))
            pairs += c.size
            decided += int(np.count_nonzero(dec))
    return pairs, decided, wrong


def boxes_scene(rng, n, centres_world, extent_scale, affine=True):
    """n boxes centred at the given world points: random rotation and scale, the box
    translated so that its centre lands on the point."""
    lower_c = np.zeros((3, n))
    e = np.exp(rng.uniform(np.log(extent_scale[0]), np.log(extent_scale[1]), (3, n)))
    lower = (lower_c - 0.5 * e).astype(np.float32)
    extent = e.astype(np.float32)
    mats = wl.random_matrices(rng, n).reshape(n, 4, 4).astype(np.float64)
    mats[:, 3, :3] = centres_world
    if not affine:
        mats[:, :3, 3] = rng.normal(0, 1e-3, (n, 3))
        mats[:, 3, 3] = rng.uniform(0.5, 2.0, n)
    return (np.ascontiguousarray(lower), np.ascontiguousarray(extent),
            np.arange(n, dtype=np.uint32), mats.reshape(n, 16).astype(np.float32))


def points_on_planes(rng, vp, n, depth_range):
    """World points on the six clip planes of vp (clip x, y or z equal to +-w)."""
    inv = np.linalg.inv(np.asarray(vp, np.float64).reshape(4, 4))
    w = np.exp(rng.uniform(np.log(depth_range[0]), np.log(depth_range[1]), n))
    clip = np.empty((n, 4))
    clip[:, 3] = w
    clip[:, :3] = rng.uniform(-1, 1, (n, 3)) * w[:, None]
    axis = rng.integers(0, 3, n)
    sign = rng.choice([-1.0, 1.0], n)
    clip[np.arange(n), axis] = sign * w
    world = clip @ inv
    return world[:, :3] / world[:, 3:4]


def test_prefilter_benchmark_views(pf):
    """The benchmark distributions (plain, stress) in every view family: never wrong, and
    it decides nearly every pair."""
    rng = np.random.default_rng(11)
    n = 60_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, 4096)
    xform = rng.integers(0, 4096, n).astype(np.uint32)
    vps = (wl.cube_face_views() + wl.stereo_views() + wl.cascade_views()
           + [wl.look_at(rng.uniform(-900, 900, 3), rng.uniform(-900, 900, 3), (0, 1, 0)) @ wl.perspective()
              for _ in range(4)])
    pairs, decided, wrong = check(pf, (lower, extent, xform, mats), vps)
    assert wrong == 0
    assert decided >= 0.98 * pairs, (decided, pairs)


def test_prefilter_camera_inside_cloud(pf):
    rng = np.random.default_rng(12)
    n = 40_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, n).reshape(n, 4, 4)
    mats[:, 3, :3] = rng.uniform(-20, 20, (n, 3))
    mats = mats.reshape(n, 16)
    scene = (lower, extent, np.arange(n, dtype=np.uint32), mats)
    vps = wl.cube_face_views() + wl.stereo_views()
    pairs, decided, wrong = check(pf, scene, vps)
    assert wrong == 0
    assert decided >= 0.6 * pairs  # boxes of 0.1-20 units within 35 units: many straddle


@pytest.mark.parametrize("scale", [(1e-7, 1e-5), (1e-4, 1e-2), (0.1, 10.0)])
def test_prefilter_boxes_on_planes(pf, scale):
    """Boxes centred exactly on the frustum planes: the rounding decides many of them."""
    rng = np.random.default_rng(13)
    n = 30_000
    vps = wl.cube_face_views() + wl.stereo_views()[:1] + wl.cascade_views()[:2]
    for vp in vps:
        pts = points_on_planes(rng, vp, n, (0.2, 4000.0))
        for affine in (True, False):
            scene = boxes_scene(rng, n, pts, scale, affine)
            _, decided, wrong = check(pf, scene, [vp])
            assert wrong == 0
            if not affine:  # projective world matrices always take the exact test
                assert decided == 0


def test_prefilter_extreme_ranges(pf):
    """Large translations, tiny and huge clip ranges, tiny boxes."""
    rng = np.random.default_rng(14)
    n = 20_000
    for trans, near, far in [(1e6, 0.1, 1e7), (1e3, 1e-5, 1e3), (1e2, 1.0, 1e9), (1e9, 1e3, 1e12)]:
        P = wl.perspective(60.0, 16 / 9, near, far)
        eye = rng.uniform(-trans, trans, 3)
        vps = [wl.look_at(eye, eye + rng.normal(size=3), (0, 1, 0)) @ P for _ in range(3)]
        for vp in vps:
            pts = points_on_planes(rng, vp, n, (near * 1.5, far * 0.9))
            for scale in [(1e-6 * trans, 1e-3 * trans), (1e-2, 1.0)]:
                _, _, wrong = check(pf, boxes_scene(rng, n, pts, scale), [vp])
                assert wrong == 0
            # and boxes spread through the volume
            pts = eye + rng.normal(0, trans, (n, 3))
            _, _, wrong = check(pf, boxes_scene(rng, n, pts, (1e-3 * trans, trans)), [vp])
            assert wrong == 0


def test_prefilter_specials(pf):
    """NaN, infinities, huge and subnormal values in boxes, matrices and views."""
    rng = np.random.default_rng(15)
    n = 20_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, n)
    specials = np.array([np.nan, np.inf, -np.inf, 3e38, -3e38, 1e-40, -1e-40, 0.0, -0.0, 2e15],
                        np.float32)
    for arr in (lower, extent, mats):
        flat = arr.reshape(-1)
        k = rng.integers(0, flat.size, flat.size // 50)
        flat[k] = rng.choice(specials, k.size)
    scene = (lower, extent, np.arange(n, dtype=np.uint32), mats)
    vps = [wl.perspective()] + wl.cube_face_views()[:2]
    bad = np.asarray(wl.perspective(), np.float32).copy().reshape(16)
    for v in specials:
        b = bad.copy()
        b[rng.integers(0, 16)] = v
        vps.append(b)
    _, _, wrong = check(pf, scene, vps)
    assert wrong == 0


def test_weak_margin_is_caught(pf_weak):
    """With the margin removed, the boxes-on-planes family exposes disagreements: the
    families above do reach the reference's rounding boundary."""
    rng = np.random.default_rng(13)
    n = 30_000
    wrong = 0
    for vp in wl.cube_face_views()[:3]:
        pts = points_on_planes(rng, vp, n, (0.2, 4000.0))
        wrong += check(pf_weak, boxes_scene(rng, n, pts, (1e-7, 1e-5)), [vp])[2]
    assert wrong > 0


def test_group_with_an_unbounded_view(pf):
    """A view that cannot be bounded (a non-finite entry) in a group: its pairs are all
    undecided, the other views of the group still decide nearly every pair."""
    rng = np.random.default_rng(16)
    n = 30_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, 2048)
    xform = rng.integers(0, 2048, n).astype(np.uint32)
    scene = (lower, extent, xform, mats)
    vps = [np.asarray(v, np.float32).reshape(16) for v in wl.cube_face_views() + wl.stereo_views()]
    vps[3] = vps[3].copy()
    vps[3][5] = np.inf
    cls = classify_group(pf, *scene, vps)
    assert np.all(cls[3] == 2)
    for k in (0, 1, 2, 4, 5, 6, 7):
        e = exact(*scene, vps[k])
        dec = cls[k] != 2
        assert not np.any(dec & ((cls[k] == 1) != e))
        assert np.count_nonzero(dec) >= 0.98 * n


def test_group_margin_is_the_largest(pf):
    """A group's decisions are never looser than any member's own: wherever a view decides
    a pair inside the group, it decides it the same way alone."""
    rng = np.random.default_rng(17)
    n = 30_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, 2048)
    xform = rng.integers(0, 2048, n).astype(np.uint32)
    scene = (lower, extent, xform, mats)
    vps = [np.asarray(v, np.float32).reshape(16)
           for v in wl.cube_face_views()[:3] + wl.cascade_views()[:3] + wl.stereo_views()]
    cls = classify_group(pf, *scene, vps)
    for k, vp in enumerate(vps):
        alone = classify(pf, *scene, vp)
        dec = cls[k] != 2
        assert np.array_equal(cls[k][dec], alone[dec])


# ---- leaving out the far plane (pf::far_plane_clear) ---------------------------------------

def _far(lib):
    lib.pf_far_scene.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 5 + [ctypes.c_size_t, ctypes.c_void_p,
                                                                            ctypes.c_void_p]
    lib.pf_far_scene.restype = None
    lib.pf_far_fuzz.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p]
    lib.pf_far_fuzz.restype = ctypes.c_int64
    return lib


def far_scene(lib, scene, vps):
    """Per view: whether the scene bound clears its z-hi plane, and the boxes for which
    that would change a decision (must be 0)."""
    lower, extent, xform, mats = [np.ascontiguousarray(a) for a in scene]
    vps = np.ascontiguousarray(np.asarray(vps, np.float32).reshape(-1, 16))
    clear = np.zeros(vps.shape[0], np.int32)
    bad = np.zeros(vps.shape[0], np.int64)
    _far(lib).pf_far_scene(lower.shape[1], lower.ctypes.data, extent.ctypes.data, xform.ctypes.data,
                           mats.ctypes.data, vps.ctypes.data, vps.shape[0], clear.ctypes.data, bad.ctypes.data)
    return clear.astype(bool), bad


def test_far_plane_left_out_for_the_stress_views(pf):
    """The stress scene (a 2^20-object chunk of it, all its shared matrices) under its cube
    faces and stereo pair, jittered: the scene lies far inside every far plane, so every
    view is cleared and the cached kernel tests five planes; every box's five-plane bits
    equal its six-plane bits."""
    sc = wl.stress_scene(n_objects=1 << 20, n_transforms=1 << 16)
    scene = (sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    rng = np.random.default_rng(21)
    for vps in (sc["vps"], [wl.jitter_view(rng, v) for v in sc["vps"]]):
        clear, bad = far_scene(pf, scene, vps)
        assert clear.all(), clear
        assert not bad.any(), bad


def test_far_plane_kept_where_it_cuts_the_scene(pf):
    """Views whose far plane passes through the scene keep it, those whose far plane lies
    past every centre leave it out, and no decision differs either way (cascades too)."""
    rng = np.random.default_rng(22)
    n = 50_000
    lower, _, extent = wl.random_boxes(rng, n)
    mats = wl.random_matrices(rng, 4096)
    xform = rng.integers(0, 4096, n).astype(np.uint32)
    scene = (lower, extent, xform, mats)
    # the centres fill [-1005, 1005]^3 and the camera looks down -z from the origin
    near_far = [wl.perspective(60.0, 16 / 9, 0.1, far) for far in (300.0, 900.0, 1004.0)]
    clear, bad = far_scene(pf, scene, near_far)
    assert not clear.any() and not bad.any()
    clear, bad = far_scene(pf, scene, wl.cascade_views())
    assert not bad.any()
    # far planes past the scene's last centre are cleared
    clear, bad = far_scene(pf, scene, [wl.perspective(60.0, 16 / 9, 0.1, far) for far in (1100.0, 5000.0)])
    assert clear.all() and not bad.any()


def test_far_plane_clear_fuzz(pf):
    """Random bounds, plane normals (unit and shorter), offsets around the bound and
    margins: wherever the test clears a plane, the bound's corners and random centres in it
    have plane values above D for every margin up to d0max."""
    viol = np.zeros(1, np.int64)
    cleared = _far(pf).pf_far_fuzz(7, 400_000, viol.ctypes.data)
    assert viol[0] == 0
    assert cleared > 50_000, cleared


def test_bound_keys_order_and_round_trip():
    """The bound keys of the Fill launch's atomicMax (the formula of pf::bound_key) keep the
    order of the floats; decoding is covered by the scene tests above."""
    import struct
    rng = np.random.default_rng(23)
    vals = np.concatenate([rng.normal(0, 1e3, 2000), rng.normal(0, 1e-30, 200), [-0.0, 0.0, 3e38, -3e38, 1e-45]])
    vals = vals.astype(np.float32)  # -0.0 before 0.0: their keys order them that way

    def key(f):
        b = struct.unpack("<I", struct.pack("<f", float(f)))[0]
        return (~b & 0xFFFFFFFF) if b & 0x80000000 else b | 0x80000000

    keys = np.array([key(v) for v in vals], np.uint64)
    order = np.argsort(vals, kind="stable")
    ks = keys[order]
    assert np.all(ks[1:] >= ks[:-1])
    assert key(-0.0) < key(0.0) < key(1e-45)


def test_tight_radius_decides_more(tmp_path):
    """On the stress distributions under the stress views, the cached boxes' radius
    leaves about a third fewer pairs undecided than the per-launch one, and decides no
    pair wrongly (the families above check correctness everywhere)."""
    loose = _build(tmp_path, "pfl")
    tight = _build(tmp_path, "pft", ["-DPF_TIGHT"])
    sc = wl.stress_scene(n_objects=1 << 17, n_transforms=1 << 14)
    scene = (sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    pairs_l, dec_l, wrong_l = check(loose, scene, sc["vps"])
    pairs_t, dec_t, wrong_t = check(tight, scene, sc["vps"])
    assert wrong_l == 0 and wrong_t == 0
    und_l, und_t = pairs_l - dec_l, pairs_t - dec_t
    assert und_t <= 0.8 * und_l, (und_l, und_t)
