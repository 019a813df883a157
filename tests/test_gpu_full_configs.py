"""The hierarchy and batched-uneven configurations at their full sizes, bit-exact against
the oracle port through the C ABI.

* Hierarchy: 4M objects over the 64k-transform tree of depth 8 (branching 2-8); three
  orbit frames, each with every local matrix replaced (an animated frame), propagated on
  the GPU (dp/transform/src/Tree.cpp:133-166) and culled through the device world
  matrices (dp/culling/cpu/src/ManagerImpl.cpp:467-518).  World matrices, dirty-world
  bits, visibility words and changed lists are compared every frame.
* Batched uneven: the 256 scenes (log-uniform 1k-1M objects, 1-6 views each) in one
  captured plan whose tuning the autotuner picks; every result's words and changed list
  against the port and against one plain launch per scene and view."""
import numpy as np
import pytest

import oracle
from conftest import f32_bits
from pipeline_gb300 import native
from pipeline_gb300 import workloads as W
from test_gpu_parity import box3_lower_extent, port_frames, setup_group

pytestmark = pytest.mark.gpu


def all_visible_words(n: int) -> np.ndarray:
    """ResultBitSet's starting state: every object visible (ResultBitSet.cpp:65-79)."""
    prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
    if n % 32:
        prev[-1] = (1 << (n % 32)) - 1
    return prev


def test_hierarchy_config_full_size(ctx):
    from pipeline_gb300.transform import Tree

    sc = W.hierarchy_scene(seed=1, frames=240)
    used = sc["n_transforms"]
    n = len(sc["xform"])
    assert n == 4_000_000 and used == 65_536
    t = Tree(ctx)
    for p, x in sc["pairs"]:
        t.add_transform(int(p), sc["locals"][x])
    t.compute()
    dev, count = t.world_device()
    lo, ex = box3_lower_extent(sc["lower"], sc["upper"])
    g = ctx.group_create()
    ctx.group_set_objects(g, lo, ex, sc["xform"])
    ctx.group_bind_device_matrices(g, dev, count)
    r = ctx.result_create(g)

    world = np.zeros((used, 16), np.float32)
    world[0] = np.eye(4, dtype=np.float32).reshape(16)
    words = (used + 31) // 32
    idx = np.arange(1, used, dtype=np.uint32)
    prev = all_visible_words(n)
    rng = np.random.default_rng(1001)
    for frame in (0, 80, 160):
        locs = W.random_matrices(rng, used)
        locs[0] = world[0]
        ctx.tree_set_locals(t.handle, idx, locs[1:])  # every transform animated
        ctx.tree_compute(t.handle)
        dirty_local = np.zeros(words + 1, np.uint32)
        dirty_local[: used // 32] = 0xFFFFFFFF
        dirty_local[0] &= ~np.uint32(1)  # the root is not updated
        dirty_world = np.zeros(words + 1, np.uint32)
        oracle.propagate(sc["pairs"], locs, world, dirty_local, dirty_world)
        assert np.array_equal(f32_bits(t.world_matrices(used)), f32_bits(world)), frame
        assert np.array_equal(t.dirty_world_matrices()[:words], dirty_world[:words]), frame

        vp = sc["vps"][frame]
        ctx.cull(g, r, vp)
        obbs = oracle.build_obbs(lo, ex, sc["xform"], world)
        bits = oracle.cull_obbs(obbs, vp, threads=16)
        del obbs
        changed = oracle.update_changed(prev, bits, n)
        assert np.array_equal(ctx.result_bits(r), bits), frame
        assert np.array_equal(ctx.result_changed(r), changed), frame
        assert 0 < len(changed) < n
    ctx.group_destroy(g)


def test_batched_config_full_size_autotuned(tmp_path, monkeypatch):
    monkeypatch.setenv("DPCULL_TUNE_CACHE", str(tmp_path / "tune.json"))  # a fresh tuning
    scenes = W.batched_scenes(seed=2)
    assert len(scenes) == 256
    n_views = sum(len(s["vps"]) for s in scenes)
    with native.Context(0) as c:
        jobs, plain = [], []
        for s in scenes:
            g = setup_group(c, s["lower"], s["upper"], s["xform"], s["mats"])
            jobs.append((g, [c.result_create(g) for _ in s["vps"]], s["vps"]))
            plain.append([c.result_create(g) for _ in s["vps"]])
        p = c.plan_create(jobs)  # no tuning given: the autotuner measures and picks one
        tuning = c.plan_tuning(p)
        assert tuning["views_per_pass"] in (1, 2, 4, 8)
        c.plan_launch(p)
        c.synchronize()
        checked = 0
        for s, (g, rs, vps), rp in zip(scenes, jobs, plain):
            for rr, vp in zip(rp, vps):
                c.cull(g, rr, vp)
            # one new result per view: each starts all visible (not consecutive frames)
            exp = [port_frames(s, [vp])[0] for vp in vps] if len(s["xform"]) < 50_000 else None
            obbs = oracle.build_obbs(s["lower"], s["extent"], s["xform"], s["mats"]) if exp is None else None
            n = len(s["xform"])
            for v, (rb, rr) in enumerate(zip(rs, rp)):
                if exp is not None:
                    bits, ch = exp[v]
                else:
                    bits = oracle.cull_obbs(obbs, vps[v], threads=16)
                    ch = oracle.update_changed(all_visible_words(n), bits, n)
                assert np.array_equal(c.result_bits(rb), bits), (checked, tuning)
                assert np.array_equal(c.result_changed(rb), ch), (checked, tuning)
                assert np.array_equal(c.result_bits(rr), bits), checked
                assert np.array_equal(c.result_changed(rr), ch), checked
                checked += 1
            del obbs
        assert checked == n_views
        c.plan_destroy(p)
