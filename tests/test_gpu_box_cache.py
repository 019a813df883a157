"""The groups' box cache (the counterpart of the reference's OBB cache,
dp/culling/cpu/src/ManagerImpl.cpp:114-162): a group culled again with unchanged objects
and matrices has its boxes stored by that cull and read from the third cull on, and every
change to the objects, the matrices or the tree its matrices are bound to makes them stale.
Every frame here is compared bit for bit with the oracle port, with the cache on and off."""
import numpy as np
import pytest

import oracle
from pipeline_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def expected(prev, lower, extent, xform, mats, vp, n):
    bits = oracle.cull_bits(lower, extent, xform, mats, vp)
    return bits, oracle.update_changed(prev, bits, n)


def all_visible(n):
    prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
    if n % 32:
        prev[-1] = (1 << (n % 32)) - 1
    return prev


@pytest.mark.parametrize("cached", [True, False])
def test_cache_follows_every_change(ctx, cached):
    """Four culls after each kind of change (objects updated, matrices updated, matrices
    replaced, objects appended, an object removed, objects replaced): the second stores the
    boxes, the third and fourth read them."""
    ctx.set_box_cache(cached)
    try:
        rng = np.random.default_rng(41)
        n, nm = 20_011, 700
        lower, _, extent = W.random_boxes(rng, n)
        mats = W.random_matrices(rng, nm)
        mats[:, 12:15] *= np.float32(0.05)
        xform = rng.integers(0, nm, n).astype(np.uint32)
        g = ctx.group_create()
        ctx.group_set_objects(g, lower, extent, xform)
        ctx.group_set_matrices(g, mats)
        r = ctx.result_create(g)
        prev = all_visible(n)
        views = [np.asarray(v, np.float32).reshape(16) for v in W.cube_face_views()[:4]]

        def frames(tag):
            for k in range(4):
                vp = views[k % len(views)]
                ctx.cull(g, r, vp)
                bits, ch = expected(prev, lower, extent, xform, mats, vp, len(xform))
                assert np.array_equal(ctx.result_bits(r), bits), (tag, k)
                assert np.array_equal(ctx.result_changed(r), ch), (tag, k)

        frames("initial")
        idx = rng.choice(n, 300, replace=False).astype(np.uint32)
        lo2, _, ex2 = W.random_boxes(rng, 300)
        xf2 = rng.integers(0, nm, 300).astype(np.uint32)
        ctx.group_update_objects(g, idx, lo2, ex2, xf2)
        lower[:, idx], extent[:, idx], xform[idx] = lo2, ex2, xf2
        frames("objects updated")
        mi = rng.choice(nm, 50, replace=False).astype(np.uint32)
        mats[mi] = W.random_matrices(rng, 50)
        mats[mi, 12:15] *= np.float32(0.05)
        ctx.group_update_matrices(g, mi, mats)
        frames("matrices updated")
        mats = W.random_matrices(rng, nm)
        mats[:, 12:15] *= np.float32(0.05)
        ctx.group_set_matrices(g, mats)
        frames("matrices replaced")
        lo3, _, ex3 = W.random_boxes(rng, 2000)
        xf3 = rng.integers(0, nm, 2000).astype(np.uint32)
        ctx.group_append_objects(g, lo3, ex3, xf3)
        lower = np.ascontiguousarray(np.concatenate([lower, lo3], axis=1))
        extent = np.ascontiguousarray(np.concatenate([extent, ex3], axis=1))
        xform = np.concatenate([xform, xf3])
        r = ctx.result_create(g)  # a new result: all visible at the group's new size
        prev = all_visible(len(xform))
        frames("objects appended")
        hole, last = 777, len(xform) - 1
        ctx.group_remove_object(g, hole)  # the last object moves into the hole
        lower[:, hole], extent[:, hole], xform[hole] = lower[:, last], extent[:, last], xform[last]
        lower, extent, xform = lower[:, :last].copy(), extent[:, :last].copy(), xform[:last].copy()
        r = ctx.result_create(g)
        prev = all_visible(len(xform))
        frames("object removed")
        lo4, _, ex4 = W.random_boxes(rng, 5003)
        xf4 = rng.integers(0, nm, 5003).astype(np.uint32)
        ctx.group_set_objects(g, lo4, ex4, xf4)
        lower, extent, xform = lo4, ex4, xf4
        r = ctx.result_create(g)
        prev = all_visible(len(xform))
        frames("objects replaced")
        ctx.group_destroy(g)
    finally:
        ctx.set_box_cache(True)


def test_cache_of_a_tree_bound_group_goes_stale_at_each_compute(ctx):
    """A group culled against a tree's device world matrices: frames with a compute (new
    local matrices) and frames without, every one against the oracle."""
    from pipeline_gb300.transform import Tree

    sc = W.hierarchy_scene(seed=6, n_objects=60_000, n_transforms=3000, frames=12)
    used = sc["n_transforms"]
    t = Tree(ctx)
    for p, x in sc["pairs"]:
        t.add_transform(int(p), sc["locals"][x])
    t.compute()
    dev, count = t.world_device()
    g = ctx.group_create()
    ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
    ctx.group_bind_device_matrices(g, dev, count)
    r = ctx.result_create(g)
    n = len(sc["xform"])
    prev = all_visible(n)
    rng = np.random.default_rng(43)
    idx = np.arange(1, used, dtype=np.uint32)
    for f in range(12):
        if f in (4, 9):  # animate: new locals, propagation on the GPU
            locs = W.random_matrices(rng, used)
            locs[0] = np.eye(4, dtype=np.float32).reshape(16)
            ctx.tree_set_locals(t.handle, idx, locs[1:])
            ctx.tree_compute(t.handle)
        world = t.world_matrices(used)
        vp = sc["vps"][f]
        ctx.cull(g, r, vp)
        bits, ch = expected(prev, sc["lower"], sc["extent"], sc["xform"], world, vp, n)
        assert np.array_equal(ctx.result_bits(r), bits), f
        assert np.array_equal(ctx.result_changed(r), ch), f
    ctx.group_destroy(g)


def test_external_device_matrices_are_never_cached(ctx):
    """Device matrices the library does not own may change behind its back: a group bound
    to them follows every change."""
    import torch

    rng = np.random.default_rng(44)
    n, nm = 30_001, 512
    lower, _, extent = W.random_boxes(rng, n)
    xform = rng.integers(0, nm, n).astype(np.uint32)
    buf = torch.zeros(nm * 16, dtype=torch.float32, device="cuda")
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_bind_device_matrices(g, buf.data_ptr(), nm)
    r = ctx.result_create(g)
    prev = all_visible(n)
    vp = np.asarray(W.cube_face_views()[0], np.float32).reshape(16)
    for f in range(6):
        mats = W.random_matrices(rng, nm)
        mats[:, 12:15] *= np.float32(0.02)
        buf.copy_(torch.from_numpy(mats.reshape(-1)))
        torch.cuda.synchronize()
        ctx.cull(g, r, vp)
        bits, ch = expected(prev, lower, extent, xform, mats, vp, n)
        assert np.array_equal(ctx.result_bits(r), bits), f
        assert np.array_equal(ctx.result_changed(r), ch), f
    ctx.group_destroy(g)
    del buf


def test_one_group_in_two_jobs_of_one_launch(ctx):
    """A group that appears in two jobs of one plan (culled without its cache) gives the
    oracle's words over several launches."""
    rng = np.random.default_rng(45)
    n, nm = 40_000, 1000
    lower, _, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, nm)
    mats[:, 12:15] *= np.float32(0.05)
    xform = rng.integers(0, nm, n).astype(np.uint32)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, mats)
    va = W.f32(W.cube_face_views()[:3])
    vb = W.f32(W.stereo_views())
    ra = [ctx.result_create(g) for _ in va]
    rb = [ctx.result_create(g) for _ in vb]
    p = ctx.plan_create([(g, ra, va), (g, rb, vb)], dict(views_per_pass=4, tiles_per_ticket=1, ctas_per_sm=0))
    for _ in range(4):
        ctx.plan_launch(p)
    for rr, vp in list(zip(ra, va)) + list(zip(rb, vb)):
        assert np.array_equal(ctx.result_bits(rr), oracle.cull_bits(lower, extent, xform, mats, vp))
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_kernel_kind_of_each_launch(ctx):
    """Which cull kernel each plan launch runs: fused after a change, the storing one on
    the next launch, the reading one from then on; the context's switch applies to a plan
    created before it; every frame is the oracle's."""
    rng = np.random.default_rng(47)
    n, nm = 50_000, 900
    lower, _, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, nm)
    mats[:, 12:15] *= np.float32(0.05)
    xform = rng.integers(0, nm, n).astype(np.uint32)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, mats)
    vps = W.f32(W.cube_face_views()[:2])
    rs = [ctx.result_create(g) for _ in vps]
    p = ctx.plan_create([(g, rs, vps)], dict(views_per_pass=2, tiles_per_ticket=1, ctas_per_sm=0))

    def launch(expect):
        before = ctx.cull_launches()
        ctx.plan_launch(p)
        after = ctx.cull_launches()
        got = [k for k in after if after[k] != before[k]]
        assert got == [expect], (got, expect)
        for r, vp in zip(rs, vps):
            assert np.array_equal(ctx.result_bits(r), oracle.cull_bits(lower, extent, xform, mats, vp))

    for kind in ("fused", "fill", "read", "read"):
        launch(kind)
    ctx.set_box_cache(False)
    try:
        launch("fused")
        launch("fused")
    finally:
        ctx.set_box_cache(True)
    launch("read")  # nothing changed while it was off
    idx = np.array([3, 77, 899], np.uint32)
    mats[idx] = W.random_matrices(rng, 3)
    ctx.group_update_matrices(g, idx, mats)
    for kind in ("fused", "fill", "read"):
        launch(kind)
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_stress_scene_cached_equals_uncached(ctx):
    """The stress distribution under 8 views over 6 launches of a plan: the words and
    changed lists with the cache (launch 2 stores it, launches 3-6 read it) equal those
    without, and the oracle's on a sample."""
    sc = W.stress_scene(seed=14, n_objects=1_000_003, n_transforms=60_000)
    rng = np.random.default_rng(46)
    frames = [np.stack([W.jitter_view(rng, v) for v in sc["vps"]]) for _ in range(6)]
    out = []
    for cached in (True, False):
        ctx.set_box_cache(cached)
        g = ctx.group_create()
        ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
        ctx.group_set_matrices(g, sc["mats"])
        rs = [ctx.result_create(g) for _ in range(8)]
        p = ctx.plan_create([(g, rs, sc["vps"])], dict(views_per_pass=8, tiles_per_ticket=1, ctas_per_sm=0))
        got = []
        for fr in frames:
            ctx.plan_set_views(p, fr)
            ctx.plan_launch(p)
            got.append([(ctx.result_bits(r).copy(), ctx.result_changed(r).copy()) for r in rs])
        out.append(got)
        ctx.plan_destroy(p)
        ctx.group_destroy(g)
    ctx.set_box_cache(True)
    for f in range(6):
        for v in range(8):
            assert np.array_equal(out[0][f][v][0], out[1][f][v][0]), (f, v)
            assert np.array_equal(out[0][f][v][1], out[1][f][v][1]), (f, v)
    m = 200_000
    obbs = oracle.build_obbs(sc["lower"][:, :m], sc["extent"][:, :m], sc["xform"][:m], sc["mats"])
    for v in range(8):
        assert np.array_equal(out[0][5][v][0][: m // 32], oracle.cull_obbs(obbs, frames[5][v], threads=8))


@pytest.mark.parametrize("far", [600.0, 1500.0])
def test_cached_views_whose_far_planes_cut_the_scene(ctx, far):
    """Cube faces beside a stereo pair at far 5000.  At far 600 the cube faces' far planes
    pass through the scene (centres within [-1005, 1005]^3), the scene bound does not
    clear them, and the cached launches keep all six planes; at far 1500 every far plane
    lies past every centre (about 500 units on), so they run five.  Either way their
    words and changed lists equal those of the uncached fused kernel (six planes) and the
    oracle's on a sample."""
    sc = W.stress_scene(seed=15, n_objects=300_007, n_transforms=20_000)
    vps = np.stack([np.asarray(v, np.float32).reshape(16)
                    for v in W.cube_face_views(far=far) + W.stereo_views()])
    rng = np.random.default_rng(47)
    frames = [np.stack([W.jitter_view(rng, v) for v in vps]) for _ in range(5)]
    out = []
    for cached in (True, False):
        ctx.set_box_cache(cached)
        g = ctx.group_create()
        ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
        ctx.group_set_matrices(g, sc["mats"])
        rs = [ctx.result_create(g) for _ in range(8)]
        p = ctx.plan_create([(g, rs, vps)], dict(views_per_pass=8, tiles_per_ticket=1, ctas_per_sm=0))
        got = []
        for fr in frames:
            ctx.plan_set_views(p, fr)
            ctx.plan_launch(p)
            got.append([(ctx.result_bits(r).copy(), ctx.result_changed(r).copy()) for r in rs])
        out.append(got)
        ctx.plan_destroy(p)
        ctx.group_destroy(g)
    ctx.set_box_cache(True)
    for f in range(5):
        for v in range(8):
            assert np.array_equal(out[0][f][v][0], out[1][f][v][0]), (f, v)
            assert np.array_equal(out[0][f][v][1], out[1][f][v][1]), (f, v)
    m = 100_000
    obbs = oracle.build_obbs(sc["lower"][:, :m], sc["extent"][:, :m], sc["xform"][:m], sc["mats"])
    for v in range(8):
        assert np.array_equal(out[0][4][v][0][: m // 32], oracle.cull_obbs(obbs, frames[4][v], threads=8))
