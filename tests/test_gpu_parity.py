"""CUDA backend against the reference: golden fixtures written by the reference itself and
the oracle port on the same seeded inputs.  Every comparison is bit-exact (visibility
words, changed lists, world matrices, bounding boxes).  All calls go through the C ABI."""
import numpy as np
import pytest

import oracle
from conftest import f32_bits, golden_scene_names, load_golden
from pipeline_gb300 import native
from pipeline_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def unpack(bits, n):
    return np.unpackbits(np.ascontiguousarray(bits, np.uint32).view(np.uint8), bitorder="little")[:n]


def extent_of(lower, upper):
    """What objectSetBoundingBox stores: Box3f(lower, upper) then upper - lower in FP32."""
    lo = np.minimum(lower, upper)  # Box3f's constructor orders the corners (non-NaN inputs)
    hi = np.maximum(lower, upper)
    nan = np.isnan(lower) | np.isnan(upper)
    lo = np.where(nan, np.float32(0), lo)
    return lo.astype(np.float32), (hi - lo).astype(np.float32)


def box3_lower_extent(lower, upper):
    """Exact Box3f(lower, upper) -> (lower, size) semantics per component, NaN included."""
    FMAX = np.float32(np.finfo(np.float32).max)
    lo = np.full(lower.shape, FMAX, np.float32)
    hi = np.full(lower.shape, -FMAX, np.float32)
    for p in (lower, upper):
        m = lo > p
        lo = np.where(m, p, lo)
        m = hi < p
        hi = np.where(m, p, hi)
    return lo.astype(np.float32), (hi - lo).astype(np.float32)


def setup_group(ctx, lower, upper, xform, mats):
    lo, ex = box3_lower_extent(np.asarray(lower, np.float32), np.asarray(upper, np.float32))
    g = ctx.group_create()
    ctx.group_set_objects(g, lo, ex, xform)
    ctx.group_set_matrices(g, mats)
    return g


@pytest.mark.parametrize("name", golden_scene_names())
def test_golden_scene(ctx, name):
    z = load_golden(name)
    n = len(z["xform"])
    g = setup_group(ctx, z["lower"], z["upper"], z["xform"], z["mats"])
    r = ctx.result_create(g)
    order = list(range(n))  # group index -> object id
    for k, vp in enumerate(z["vps"]):
        ctx.cull(g, r, vp)
        ch = ctx.result_changed(r)
        assert np.array_equal(np.asarray(order)[ch], z[f"changed{k}"]), (name, k)
        assert np.array_equal(ctx.result_bits(r), z[f"bits{k}"]), (name, k)
    lo, hi = ctx.group_bounding_box(g)
    assert np.array_equal(f32_bits(np.concatenate([lo, hi])), f32_bits(z["bbox"])), name
    for o in z["removals"]:
        hole = order.index(int(o))
        ctx.group_remove_object(g, hole)
        order[hole] = order[-1]
        order.pop()
    if len(z["removals"]) or len(z["dirty"]):
        ctx.cull(g, r, z["vps"][0])
        assert np.array_equal(np.asarray(order, np.int32), z["order_after"])
        ch = ctx.result_changed(r)
        assert np.array_equal(np.asarray(order)[ch], z["changed_after"]), name
        assert np.array_equal(ctx.result_bits(r), z["bits_after"]), name
    ctx.group_destroy(g)


def test_golden_tree(ctx):
    from pipeline_gb300.transform import Tree

    z = load_golden("tree_small.npz")
    pairs, locs = z["pairs"], z["locals"]
    used = locs.shape[0]
    words = (used + 31) // 32
    t = Tree(ctx)
    for p, x in pairs:
        assert t.add_transform(int(p), locs[x]) == x
    t.compute()
    assert np.array_equal(f32_bits(t.world_matrices(used)), f32_bits(z["world0"]))
    assert np.array_equal(t.dirty_world_matrices()[:words], z["dirty0"])
    for k, i in enumerate(z["upd"]):
        t.update_local_matrix(int(i), z["upd_locals"][k])
    t.compute()
    assert np.array_equal(f32_bits(t.world_matrices(used)), f32_bits(z["world1"]))
    assert np.array_equal(t.dirty_world_matrices()[:words], z["dirty1"])
    victim = int(z["victim"])
    new_parent = int(pairs[z["level_offsets"][2]][1])
    t.remove_transform(victim)
    assert t.add_transform(new_parent, locs[victim]) == victim
    for i in range(1, used):
        t.update_local_matrix(i, locs[i])
    t.compute()
    assert np.array_equal(f32_bits(t.world_matrices(used)), f32_bits(z["world2"]))
    assert np.array_equal(t.dirty_world_matrices()[:words], z["dirty2"])


def port_frames(sc, vps):
    """Bits and changed lists of consecutive culls, from the oracle port."""
    n = len(sc["xform"])
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
    if n % 32:
        prev[-1] = (1 << (n % 32)) - 1
    out = []
    for vp in vps:
        bits = oracle.cull_obbs(obbs, vp, threads=8)
        ch = oracle.update_changed(prev, bits, n)
        out.append((bits, ch))
    return out


def test_plain_config_full_size(ctx):
    """100k objects, own matrices, two frames with a 1 degree yaw (the plain configuration)."""
    sc = W.plain_scene(0, 100_000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    r = ctx.result_create(g)
    exp = port_frames(sc, sc["vps"])
    for vp, (bits, ch) in zip(sc["vps"], exp):
        ctx.cull(g, r, vp)
        assert np.array_equal(ctx.result_bits(r), bits)
        assert np.array_equal(ctx.result_changed(r), ch)
    assert len(exp[1][1]) > 0  # the yaw changes some objects
    ctx.group_destroy(g)


def test_result_read_one_call(ctx):
    """dpcull_result_read returns the same words and changed list as the two separate
    reads, over frames whose changed lists grow past the copied prefix and shrink again."""
    sc = W.plain_scene(0, 100_000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    r = ctx.result_create(g)
    rng = np.random.default_rng(8)
    vps = [sc["vps"][0], sc["vps"][1]] + [W.jitter_view(rng, sc["vps"][0], 30.0) for _ in range(3)] + [sc["vps"][0]]
    exp = port_frames(sc, vps)
    bits = np.zeros(3125, np.uint32)
    changed = np.zeros(100_000, np.uint32)
    for vp, (eb, ec) in zip(vps, exp):
        ctx.cull(g, r, vp)
        n = ctx.result_read(r, bits, changed)
        assert np.array_equal(bits, eb)
        assert n == len(ec) and np.array_equal(changed[:n], ec)
    assert max(len(ec) for _, ec in exp) > 4096  # some frame needed the second copy
    ctx.cull(g, r, vps[1])  # the 1 degree yaw after the first frame again
    assert len(exp[1][1]) > 1
    with pytest.raises(native.DpcullError) as e:
        ctx.result_read(r, bits, np.zeros(1, np.uint32))
    assert e.value.code == native.ERR_CAPACITY
    ctx.group_destroy(g)


@pytest.mark.parametrize("n", [0, 1, 31, 32, 33, 1023, 1024, 1025, 4097, 70001])
def test_ragged_sizes(ctx, n):
    rng = np.random.default_rng(n)
    lower, upper, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, max(n // 3, 1))
    mats[:, 12:15] *= np.float32(0.02)
    xform = rng.integers(0, mats.shape[0], n, dtype=np.uint32)
    sc = dict(lower=lower, extent=extent, xform=xform, mats=mats)
    vps = W.f32(W.cube_face_views()[:3])
    g = setup_group(ctx, lower, upper, xform, mats)
    r = ctx.result_create(g)
    for vp, (bits, ch) in zip(vps, port_frames(sc, vps)):
        ctx.cull(g, r, vp)
        assert np.array_equal(ctx.result_bits(r), bits[: (n + 31) // 32])
        assert np.array_equal(ctx.result_changed(r), ch)
    ctx.group_destroy(g)


def test_batched_equals_plain_and_port(ctx):
    """Uneven scenes x 1-6 views in one persistent launch == per-view plain launches == port."""
    scenes = W.batched_scenes(seed=7, n_scenes=10, nmin=500, nmax=60_000)
    jobs, plain, exp = [], [], []
    for s in scenes:
        g = setup_group(ctx, s["lower"], s["upper"], s["xform"], s["mats"])
        rs = [ctx.result_create(g) for _ in s["vps"]]
        jobs.append((g, rs, s["vps"]))
        rp = [ctx.result_create(g) for _ in s["vps"]]
        plain.append((g, rp, s["vps"]))
        exp.append([port_frames(s, [vp])[0] for vp in s["vps"]])
    for tuning in (None, dict(views_per_pass=1, tiles_per_ticket=1, ctas_per_sm=1),
                   dict(views_per_pass=2, tiles_per_ticket=4, ctas_per_sm=2),
                   dict(views_per_pass=8, tiles_per_ticket=2, ctas_per_sm=0)):
        # fresh results each round: reset by culling through new results
        jobs_t = [(g, [ctx.result_create(g) for _ in vps], vps) for g, _, vps in jobs]
        ctx.cull_batched(jobs_t, tuning)
        for (g, rs, vps), e in zip(jobs_t, exp):
            for r, (bits, ch) in zip(rs, e):
                assert np.array_equal(ctx.result_bits(r), bits), tuning
                assert np.array_equal(ctx.result_changed(r), ch), tuning
    for (g, rp, vps), e in zip(plain, exp):
        for r, vp, (bits, ch) in zip(rp, vps, e):
            ctx.cull(g, r, vp)
            assert np.array_equal(ctx.result_bits(r), bits)
            assert np.array_equal(ctx.result_changed(r), ch)
    for g, _, _ in jobs:
        ctx.group_destroy(g)


def test_plan_graph_frames(ctx):
    """A captured plan replayed over several camera frames (double-buffered view upload)."""
    sc = W.stress_scene(seed=9, n_objects=300_000, n_transforms=20_000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    rs = [ctx.result_create(g) for _ in range(8)]
    p = ctx.plan_create([(g, rs, sc["vps"])], dict(views_per_pass=4, tiles_per_ticket=2, ctas_per_sm=0))
    rng = np.random.default_rng(3)
    frames = [sc["vps"]] + [np.stack([W.jitter_view(rng, v) for v in sc["vps"]]) for _ in range(4)]
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    n = 300_000
    prev = [np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32) for _ in range(8)]
    out_bits = [np.zeros((n + 31) // 32, np.uint32) for _ in range(8)]
    out_changed = [np.zeros(n, np.uint32) for _ in range(8)]
    for vps in frames:
        ctx.plan_set_views(p, vps)
        ctx.plan_launch(p)
        n_ch = ctx.plan_read(p, out_bits, out_changed)  # every result in two waits
        for v in range(8):
            bits = oracle.cull_obbs(obbs, vps[v], threads=8)
            ch = oracle.update_changed(prev[v], bits, n)
            assert np.array_equal(ctx.result_bits(rs[v]), bits)
            assert np.array_equal(ctx.result_changed(rs[v]), ch)
            assert np.array_equal(out_bits[v], bits)
            assert n_ch[v] == len(ch) and np.array_equal(out_changed[v][: len(ch)], ch)
    # a plan without set_views replays its last matrices
    ctx.plan_launch(p)
    for v in range(8):
        assert len(ctx.result_changed(rs[v])) == 0
    # the cull kernel's own duration, from events inside the graph, for both kept launches
    k0, k1 = ctx.plan_kernel_ms(p, 0), ctx.plan_kernel_ms(p, 1)
    assert 0.0 < k0 < 1000.0 and 0.0 < k1 < 1000.0
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_plan_snapshot_pipelined_frames(ctx):
    """The pipelined frame loop: frame i-1 is snapshotted before frame i is launched and
    read while frame i culls.  Every frame's words and changed lists reach the host
    bit-exact, although the results on the device already hold the next frame."""
    sc = W.stress_scene(seed=12, n_objects=250_001, n_transforms=10_000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    nv = 6
    rs = [ctx.result_create(g) for _ in range(nv)]
    p = ctx.plan_create([(g, rs, sc["vps"][:nv])], dict(views_per_pass=8, tiles_per_ticket=1, ctas_per_sm=0))
    rng = np.random.default_rng(5)
    frames = [sc["vps"][:nv]] + [np.stack([W.jitter_view(rng, v) for v in sc["vps"][:nv]]) for _ in range(5)]
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    n = 250_001
    expect = []
    prev = [np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32) for _ in range(nv)]
    prev = [np.where(np.arange(len(w)) == len(w) - 1, (1 << (n % 32)) - 1, w).astype(np.uint32) for w in prev]
    for vps in frames:
        fr = []
        for v in range(nv):
            bits = oracle.cull_obbs(obbs, vps[v], threads=8)
            fr.append((bits, oracle.update_changed(prev[v], bits, n)))
        expect.append(fr)
    out_bits = [np.zeros((n + 31) // 32, np.uint32) for _ in range(nv)]
    out_changed = [np.zeros(n, np.uint32) for _ in range(nv)]

    def check(k, n_ch):
        for v in range(nv):
            bits, ch = expect[k][v]
            assert np.array_equal(out_bits[v], bits), (k, v)
            assert n_ch[v] == len(ch) and np.array_equal(out_changed[v][: len(ch)], ch), (k, v)

    for i, vps in enumerate(frames):
        ctx.plan_set_views(p, vps)
        if i:
            ctx.plan_snapshot(p)
        ctx.plan_launch(p)
        if i:
            ctx.plan_read_wait(p)
            n_ch = ctx.plan_read_async(p, out_bits, out_changed)
            ctx.plan_read_wait(p)
            check(i - 1, n_ch)
    n_ch = ctx.plan_read_async(p, out_bits, out_changed)  # no snapshot pending: the last launch
    ctx.plan_read_wait(p)
    check(len(frames) - 1, n_ch)
    # the device results hold the last frame
    for v in range(nv):
        assert np.array_equal(ctx.result_bits(rs[v]), expect[-1][v][0])
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_plan_read_between_snapshot_and_async_read(ctx):
    """snapshot of frame 0, launch of frame 1, dpcull_plan_read (frame 1), then
    dpcull_plan_read_async: the blocking read returns frame 1 and the asynchronous read
    still returns the snapshot of frame 0, words and changed lists with their own counts."""
    n, nv = 100_003, 4
    sc = W.stress_scene(seed=13, n_objects=n, n_transforms=5000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    rs = [ctx.result_create(g) for _ in range(nv)]
    p = ctx.plan_create([(g, rs, sc["vps"][:nv])], dict(views_per_pass=4, tiles_per_ticket=1, ctas_per_sm=0))
    rng = np.random.default_rng(14)
    f0 = sc["vps"][:nv]
    f1 = np.stack([W.jitter_view(rng, v, 25.0) for v in f0])
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    prev = [np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32) for _ in range(nv)]
    for w in prev:
        w[-1] = (1 << (n % 32)) - 1
    expect = []
    for vps in (f0, f1):
        fr = []
        for v in range(nv):
            bits = oracle.cull_obbs(obbs, vps[v], threads=8)
            fr.append((bits, oracle.update_changed(prev[v], bits, n)))
        expect.append(fr)
    assert any(len(expect[0][v][1]) != len(expect[1][v][1]) for v in range(nv))
    bits0 = [np.zeros((n + 31) // 32, np.uint32) for _ in range(nv)]
    ch0 = [np.zeros(n, np.uint32) for _ in range(nv)]
    bits1 = [np.zeros((n + 31) // 32, np.uint32) for _ in range(nv)]
    ch1 = [np.zeros(n, np.uint32) for _ in range(nv)]
    ctx.plan_set_views(p, f0)
    ctx.plan_launch(p)
    ctx.plan_snapshot(p)
    ctx.plan_set_views(p, f1)
    ctx.plan_launch(p)
    n1 = ctx.plan_read(p, bits1, ch1)
    n0 = ctx.plan_read_async(p, bits0, ch0)
    ctx.plan_read_wait(p)
    for k, (nk, bk, ck) in enumerate(((n0, bits0, ch0), (n1, bits1, ch1))):
        for v in range(nv):
            eb, ec = expect[k][v]
            assert np.array_equal(bk[v], eb), (k, v)
            assert nk[v] == len(ec) and np.array_equal(ck[v][: len(ec)], ec), (k, v)
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_plan_snapshot_held_across_launches(ctx):
    """Launches write their results into their slot's copy buffer once asynchronous reads
    are in use.  A snapshot that is still unread when its slot is launched again keeps its
    buffer (that launch skips its copies), a snapshot of a launch without copies copies the
    live results, and every read returns the frame it snapshotted, against the port."""
    n, nv = 70_001, 3
    sc = W.stress_scene(seed=21, n_objects=n, n_transforms=3000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    rs = [ctx.result_create(g) for _ in range(nv)]
    p = ctx.plan_create([(g, rs, sc["vps"][:nv])], dict(views_per_pass=4, tiles_per_ticket=1, ctas_per_sm=0))
    rng = np.random.default_rng(22)
    frames = [np.stack([W.jitter_view(rng, v, 20.0) for v in sc["vps"][:nv]]) for _ in range(6)]
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    prev = [np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32) for _ in range(nv)]
    for w in prev:
        w[-1] = (1 << (n % 32)) - 1
    expect = []
    for vps in frames:
        fr = []
        for v in range(nv):
            bits = oracle.cull_obbs(obbs, vps[v], threads=8)
            fr.append((bits, oracle.update_changed(prev[v], bits, n)))
        expect.append(fr)

    def launch(k):
        ctx.plan_set_views(p, frames[k])
        ctx.plan_launch(p)

    def read_and_check(k):
        bits = [np.zeros((n + 31) // 32, np.uint32) for _ in range(nv)]
        ch = [np.zeros(n, np.uint32) for _ in range(nv)]
        cnt = ctx.plan_read_async(p, bits, ch)
        ctx.plan_read_wait(p)
        for v in range(nv):
            eb, ec = expect[k][v]
            assert np.array_equal(bits[v], eb), (k, v)
            assert cnt[v] == len(ec) and np.array_equal(ch[v][: len(ec)], ec), (k, v)

    launch(0)
    ctx.plan_snapshot(p)        # frame 0 was launched without copies: copied from the results
    launch(1)                   # writes its copies
    read_and_check(0)
    ctx.plan_snapshot(p)        # frame 1, from its copies
    launch(2)
    launch(3)                   # the slot of the unread snapshot: no copies this time
    read_and_check(1)
    ctx.plan_snapshot(p)        # frame 3 has no copies: copied from the results
    read_and_check(3)
    launch(4)
    read_and_check(4)           # no pending snapshot: one of the last launch
    ctx.plan_snapshot(p)
    launch(5)
    read_and_check(4)
    read_and_check(5)
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_plan_autotuned(ctx, tmp_path, monkeypatch):
    sc = W.stress_scene(seed=10, n_objects=200_000, n_transforms=5000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    rs = [ctx.result_create(g) for _ in range(8)]
    p = ctx.plan_create([(g, rs, sc["vps"])])
    t = ctx.plan_tuning(p)
    assert t["views_per_pass"] in (1, 2, 4, 8)
    ctx.plan_launch(p)
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    for v in range(8):
        assert np.array_equal(ctx.result_bits(rs[v]), oracle.cull_obbs(obbs, sc["vps"][v], 8))
    ctx.plan_destroy(p)
    ctx.group_destroy(g)


def test_hierarchy_propagate_then_cull(ctx):
    """Tree propagation on the GPU feeding the cull through device-bound world matrices."""
    from pipeline_gb300.transform import Tree

    sc = W.hierarchy_scene(seed=4, n_objects=400_000, frames=3)
    t = Tree(ctx)
    for p, x in sc["pairs"]:
        t.add_transform(int(p), sc["locals"][x])
    t.compute()
    used = sc["n_transforms"]
    # oracle: the same propagation on arrays
    world = np.zeros((used, 16), np.float32)
    world[0] = np.eye(4, dtype=np.float32).reshape(16)
    dl = np.zeros((used + 31) // 32 + 1, np.uint32)
    dl[:] = 0xFFFFFFFF
    dw = np.zeros_like(dl)
    oracle.propagate(sc["pairs"], sc["locals"], world, dl, dw)
    assert np.array_equal(f32_bits(t.world_matrices(used)), f32_bits(world))
    dev, count = t.world_device()
    g = ctx.group_create()
    lo, ex = box3_lower_extent(sc["lower"], sc["upper"])
    ctx.group_set_objects(g, lo, ex, sc["xform"])
    ctx.group_bind_device_matrices(g, dev, count)
    r = ctx.result_create(g)
    s = dict(lower=lo, extent=ex, xform=sc["xform"], mats=world)
    for vp, (bits, ch) in zip(sc["vps"], port_frames(s, sc["vps"])):
        ctx.cull(g, r, vp)
        assert np.array_equal(ctx.result_bits(r), bits)
        assert np.array_equal(ctx.result_changed(r), ch)
    ctx.group_destroy(g)


@pytest.mark.parametrize("offset_floats", [0, 4, 8, 12])
def test_bound_matrices_any_16_byte_alignment(ctx, offset_floats):
    """Device-bound matrix arrays need only 16-byte alignment: the 32-byte aligned ones
    (offsets 0 and 8 floats) take the 256-bit matrix loads, the others the 128-bit ones;
    both are bit-exact against the oracle, in the plain and the batched launch."""
    import torch

    rng = np.random.default_rng(21)
    n, n_mats = 70_001, 4096
    lower, _, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, n_mats)
    xform = rng.integers(0, n_mats, n).astype(np.uint32)
    buf = torch.zeros(n_mats * 16 + 16, dtype=torch.float32, device="cuda")
    view = buf[offset_floats: offset_floats + n_mats * 16]
    view.copy_(torch.from_numpy(np.ascontiguousarray(mats).reshape(-1)))
    torch.cuda.synchronize()
    assert view.data_ptr() % 32 == (0 if offset_floats % 8 == 0 else 16)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_bind_device_matrices(g, view.data_ptr(), n_mats)
    vps = W.cube_face_views()[:3] + W.stereo_views()
    exp = port_frames(dict(lower=lower, extent=extent, xform=xform, mats=mats), vps)
    r = ctx.result_create(g)
    for vp, (bits, ch) in zip(vps, exp):
        ctx.cull(g, r, vp)
        assert np.array_equal(ctx.result_bits(r), bits)
        assert np.array_equal(ctx.result_changed(r), ch)
    rs = [ctx.result_create(g) for _ in vps]
    ctx.cull_batched([(g, rs, vps)])
    for rv, (bits, _) in zip(rs, exp):
        assert np.array_equal(ctx.result_bits(rv), bits)
    # one launch over this group and a group with its own (aligned) copy of the matrices:
    # the launch takes the 256-bit loads only when both arrays allow them
    g2 = ctx.group_create()
    ctx.group_set_objects(g2, lower, extent, xform)
    ctx.group_set_matrices(g2, mats)
    rs1 = [ctx.result_create(g) for _ in vps]
    rs2 = [ctx.result_create(g2) for _ in vps]
    ctx.cull_batched([(g, rs1, vps), (g2, rs2, vps)])
    for r1, r2, (bits, _) in zip(rs1, rs2, exp):
        assert np.array_equal(ctx.result_bits(r1), bits)
        assert np.array_equal(ctx.result_bits(r2), bits)
    ctx.group_destroy(g2)
    ctx.group_destroy(g)
    del buf


def test_stress_full_size_eight_views(ctx):
    """16M objects over 1M shared transforms, 8 views, one batched launch: every visibility
    word of every view equals the oracle's (multi-threaded port)."""
    sc = W.stress_scene()
    n = len(sc["xform"])
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    rs = [ctx.result_create(g) for _ in range(8)]
    ctx.cull_batched([(g, rs, sc["vps"])])
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    for v in range(8):
        bits = oracle.cull_obbs(obbs, sc["vps"][v], threads=16)
        assert np.array_equal(ctx.result_bits(rs[v]), bits), v
        ch = ctx.result_changed(rs[v])
        # first cull: changed = invisible objects, ascending
        vis = unpack(bits, n)
        assert np.array_equal(ch, np.flatnonzero(vis == 0))
    del obbs
    ctx.group_destroy(g)


def test_large_group_repeating_pattern(ctx):
    """2^28 + 37 objects: a 2^20-object pattern repeated, with a ragged tail.  Checks the
    index, word and chunk arithmetic at scale through properties that hold at any size:
    the visibility words repeat with the pattern's period and the first period equals the
    oracle's; a second frame's changed list is the pattern's list shifted by every period;
    the batched launch over two views agrees with the plain one."""
    P, reps, tail = 1 << 20, 256, 37
    n = P * reps + tail
    rng = np.random.default_rng(23)
    lower_p, _, extent_p = W.random_boxes(rng, P)
    mats = W.random_matrices(rng, 4096)
    xform_p = rng.integers(0, 4096, P).astype(np.uint32)
    idx = np.arange(n, dtype=np.int64) % P
    g = ctx.group_create()
    ctx.group_set_objects(g, lower_p[:, idx], extent_p[:, idx], xform_p[idx])
    del idx
    ctx.group_set_matrices(g, mats)
    vps = [W.f32([W.perspective()])[0], W.f32([W.rot_y(1.0) @ W.perspective()])[0]]
    exp = port_frames(dict(lower=lower_p, extent=extent_p, xform=xform_p, mats=mats), vps)
    wp = P // 32
    r = ctx.result_create(g)
    bits = np.zeros((n + 31) // 32, np.uint32)
    changed = np.zeros(n, np.uint32)
    for k, vp in enumerate(vps):
        ctx.cull(g, r, vp)
        m = ctx.result_read(r, bits, changed)
        pb, pc = exp[k]
        assert np.array_equal(bits[: wp * reps].reshape(reps, wp), np.broadcast_to(pb, (reps, wp))), k
        # the 37 tail objects: one whole word and 5 bits of the last, whose padding is clear
        assert bits[wp * reps] == pb[0], k
        assert bits[wp * reps + 1] == (pb[1] & np.uint32(0x1F)), k
        if k == 1:  # the changed list: every period's changes, then the tail's
            want = np.concatenate([pc.astype(np.int64) + j * P for j in range(reps)] +
                                  [pc[pc < tail].astype(np.int64) + reps * P])
            assert m == want.size and np.array_equal(changed[:m].astype(np.int64), want)
    rs = [ctx.result_create(g) for _ in vps]
    ctx.cull_batched([(g, rs, vps)])
    for rv, vp_bits in zip(rs, [exp[0][0], exp[1][0]]):
        b = ctx.result_bits(rv)
        assert np.array_equal(b[: wp * reps].reshape(reps, wp), np.broadcast_to(vp_bits, (reps, wp)))
    ctx.group_destroy(g)


def test_bad_transform_index_is_an_error(ctx):
    rng = np.random.default_rng(1)
    lower, upper, extent = W.random_boxes(rng, 100)
    xform = np.arange(100, dtype=np.uint32)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, W.random_matrices(rng, 50))
    r = ctx.result_create(g)
    with pytest.raises(native.DpcullError) as e:
        ctx.cull(g, r, W.f32([W.perspective()])[0])
    assert e.value.code == native.ERR_OUT_OF_RANGE
    g2 = ctx.group_create()
    with pytest.raises(native.DpcullError):
        ctx.cull(g2, r, W.f32([W.perspective()])[0])  # result of another group
    ctx.group_destroy(g)
    ctx.group_destroy(g2)


def test_object_updates_and_appends(ctx):
    rng = np.random.default_rng(2)
    n = 5000
    lower, upper, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, 100)
    mats[:, 12:15] *= np.float32(0.01)
    xform = rng.integers(0, 100, n, dtype=np.uint32)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, mats)
    r = ctx.result_create(g)
    vp = W.f32(W.cube_face_views())[4]
    ctx.cull(g, r, vp)
    # move some objects, append some, update some matrices in place
    idx = rng.choice(n, 300, replace=False).astype(np.uint32)
    l2, u2, e2 = W.random_boxes(rng, 300)
    x2 = rng.integers(0, 100, 300, dtype=np.uint32)
    ctx.group_update_objects(g, idx, l2, e2, x2)
    lower[:, idx], extent[:, idx], xform[idx] = l2, e2, x2
    l3, u3, e3 = W.random_boxes(rng, 77)
    x3 = rng.integers(0, 100, 77, dtype=np.uint32)
    ctx.group_append_objects(g, l3, e3, x3)
    lower, extent, xform = np.c_[lower, l3], np.c_[extent, e3], np.r_[xform, x3]
    mi = np.array([3, 50, 99], np.uint32)
    mats[mi] = W.random_matrices(rng, 3)
    ctx.group_update_matrices(g, mi, mats)
    prev = ctx.result_bits(r).copy()
    ctx.cull(g, r, vp)
    bits = oracle.cull_bits(lower, extent, xform, mats, vp)
    assert np.array_equal(ctx.result_bits(r), bits)
    # appended objects start visible (ResultBitSet resize), others compare with prev
    m = n + 77
    pv = np.zeros((m + 31) // 32, np.uint32)
    pv[: prev.shape[0]] = prev
    for i in range(n, m):
        pv[i // 32] |= np.uint32(1 << (i % 32))
    assert np.array_equal(ctx.result_changed(r), oracle.changed_list(pv, bits, m))
    ctx.group_destroy(g)


def near_plane_scene(seed: int, n: int, vp: np.ndarray):
    """Tiny boxes centred on the frustum's boundary planes of `vp` (and on the extended
    planes outside it), the worst case for the prefilter's error margins."""
    rng = np.random.default_rng(seed)
    M = np.asarray(vp, np.float64).reshape(4, 4)
    Minv = np.linalg.inv(M)
    ndc = rng.uniform(-1.3, 1.3, (n, 3))
    axis = rng.integers(0, 3, n)
    side = rng.choice([-1.0, 1.0], n)
    ndc[np.arange(n), axis] = side * (1.0 + rng.choice([0.0, 1e-7, -1e-7, 1e-5, -1e-5, 1e-3], n))
    w = rng.uniform(0.2, 3000.0, n)
    clip = np.c_[ndc * w[:, None], w]
    world = clip @ Minv
    world = world[:, :3] / world[:, 3:4]
    size = 10.0 ** rng.uniform(-6, 0.5, (3, n))
    lower = (world.T - size / 2).astype(np.float32)
    upper = (world.T + size / 2).astype(np.float32)
    ident = np.eye(4, dtype=np.float32).reshape(1, 16)
    mats = np.repeat(ident, 4, axis=0)
    mats[1, 12:15] = [1e-3, 0, 0]
    mats[2, :3] = [0.999999, 1e-4, 0]
    mats[3, 3] = 1e-6  # projective
    xform = rng.integers(0, 4, n, dtype=np.uint32)
    return lower, upper, xform, mats


@pytest.mark.parametrize("prefilter", [True, False])
def test_prefilter_is_exact_near_planes(ctx, prefilter):
    views = W.f32([W.perspective(), W.cube_face_views()[0], W.cascade_views()[1],
                   W.stereo_views()[1], W.perspective(90.0, 1.0, 0.5, 100.0)])
    for s, vp in enumerate(views):
        lower, upper, xform, mats = near_plane_scene(50 + s, 40_000, vp)
        lo, ex = box3_lower_extent(lower, upper)
        g = ctx.group_create()
        ctx.group_set_objects(g, lo, ex, xform)
        ctx.group_set_matrices(g, mats)
        ctx.set_prefilter(prefilter)
        rs = [ctx.result_create(g) for _ in range(len(views))]
        ctx.cull_batched([(g, rs, views)], dict(views_per_pass=8, tiles_per_ticket=1, ctas_per_sm=0))
        r1 = ctx.result_create(g)
        ctx.cull(g, r1, vp)
        ctx.set_prefilter(True)
        exp = oracle.cull_bits(lo, ex, xform, mats, vp)
        assert np.array_equal(ctx.result_bits(r1), exp), (s, prefilter)
        for r, v2 in zip(rs, views):
            assert np.array_equal(ctx.result_bits(r), oracle.cull_bits(lo, ex, xform, mats, v2)), (s, prefilter)
        ctx.group_destroy(g)


def test_prefilter_equals_exact_on_golden_specials(ctx):
    z = load_golden("scene_specials.npz")
    lo, ex = box3_lower_extent(z["lower"], z["upper"])
    g = ctx.group_create()
    ctx.group_set_objects(g, lo, ex, z["xform"])
    ctx.group_set_matrices(g, z["mats"])
    out = {}
    for pf in (True, False):
        ctx.set_prefilter(pf)
        rs = [ctx.result_create(g) for _ in z["vps"]]
        ctx.cull_batched([(g, rs, z["vps"])])
        out[pf] = [ctx.result_bits(r) for r in rs]
    ctx.set_prefilter(True)
    for a, b, k in zip(out[True], out[False], range(len(z["vps"]))):
        assert np.array_equal(a, b)
        assert np.array_equal(a, z[f"bits{k}"])  # visibility depends on the view only
    ctx.group_destroy(g)


def test_kernel_launch_counter(ctx):
    sc = W.plain_scene(5, 5000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    r = ctx.result_create(g)
    before = ctx.kernel_launches
    ctx.cull(g, r, sc["vps"][0])
    ctx.synchronize()
    assert ctx.kernel_launches > before
    ctx.group_destroy(g)


def test_plan_read_empty_group_and_capacity(ctx):
    """dpcull_plan_read over a plan whose jobs include an empty group: results come back in
    job and view order (the empty group's list is empty), and a changed-list buffer that is
    too small is reported as DPCULL_ERR_CAPACITY."""
    from pipeline_gb300 import native

    sc = W.stress_scene(seed=21, n_objects=50_000, n_transforms=2000)
    g = setup_group(ctx, sc["lower"], sc["upper"], sc["xform"], sc["mats"])
    empty = ctx.group_create()
    ctx.group_set_objects(empty, np.zeros((3, 0), np.float32), np.zeros((3, 0), np.float32),
                          np.zeros(0, np.uint32))
    ctx.group_set_matrices(empty, sc["mats"])
    r0 = [ctx.result_create(empty)]
    rs = [ctx.result_create(g) for _ in range(3)]
    vps = sc["vps"][:3]
    p = ctx.plan_create([(empty, r0, vps[:1]), (g, rs, vps)], dict(views_per_pass=4, tiles_per_ticket=1, ctas_per_sm=0))
    ctx.plan_launch(p)
    n = 50_000
    bits = [None] + [np.zeros((n + 31) // 32, np.uint32) for _ in range(3)]
    changed = [None] + [np.zeros(n, np.uint32) for _ in range(3)]
    n_ch = ctx.plan_read(p, bits, changed)
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    all_ones = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)  # a first cull: all visible
    all_ones[-1] = (1 << (n % 32)) - 1 if n % 32 else 0xFFFFFFFF  # objects 0..n-1 only
    assert n_ch[0] == 0
    for v in range(3):
        want = oracle.cull_obbs(obbs, vps[v], threads=8)
        ch = oracle.update_changed(all_ones.copy(), want, n)
        assert np.array_equal(bits[v + 1], want)
        assert n_ch[v + 1] == len(ch) and np.array_equal(changed[v + 1][: len(ch)], ch)
    # the same through the asynchronous read, overlapped with the next launch
    abits = [None] + [np.zeros((n + 31) // 32, np.uint32) for _ in range(3)]
    achanged = [None] + [np.zeros(n, np.uint32) for _ in range(3)]
    a_ch = ctx.plan_read_async(p, abits, achanged)
    prev = [b.copy() for b in bits[1:]]
    ctx.plan_set_views(p, np.stack([W.jitter_view(np.random.default_rng(5), v) for v in vps]))
    ctx.plan_launch(p)  # runs while the copies land; must not disturb them
    ctx.plan_read_wait(p)
    assert np.array_equal(a_ch, n_ch)
    for v in range(3):
        assert np.array_equal(abits[v + 1], prev[v])
        assert np.array_equal(achanged[v + 1][: n_ch[v + 1]], changed[v + 1][: n_ch[v + 1]])
    # a buffer too small for a changed list
    small = [None] + [np.zeros(1, np.uint32) for _ in range(3)]
    if int(n_ch[1:].max()) > 1:
        with pytest.raises(native.DpcullError):
            ctx.plan_read(p, [None] * 4, small)
    ctx.plan_destroy(p)
    ctx.group_destroy(g)
    ctx.group_destroy(empty)
