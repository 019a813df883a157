"""Writes the golden culling fixtures in this directory from the reference itself.

The reference has no culling or transform tests and no golden vectors, so these are
produced by running the reference's own CPU manager and transform tree (compiled from
the reference sources by oracle/Makefile into oracle/_ref/libdpref.so) on seeded inputs.
The C restatement (oracle/_build/liborc.so) is checked against them in
tests/test_oracle_golden.py, and the CUDA backend in tests/test_gpu_parity.py.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from pipeline_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent


def words(n: int) -> int:
    return (n + 31) // 32


def special_floats(rng, shape, frac=0.02):
    """Random finite values with a fraction of specials (NaN, +-inf, +-0, subnormals, huge)."""
    x = rng.uniform(-20, 20, shape).astype(np.float32)
    pool = np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 1e-40, -1e-40, 3e38, -3e38, 1e-30],
                    np.float32)
    m = rng.random(shape) < frac
    x[m] = rng.choice(pool, m.sum())
    return x


def scene_case(R, lower, upper, xform, mats, vps, removals=(), dirty=()):
    """Runs cull for every vp, then removals + cull(vps[0]), recording everything."""
    m = R.manager()
    g = m.group()
    r = m.result(g)
    n = len(xform)
    m.add_boxes(g, lower, upper, xform)
    m.set_matrices(g, mats)
    out = {}
    for k, vp in enumerate(vps):
        m.cull(g, r, vp)
        out[f"changed{k}"] = m.changed(r).astype(np.int32)
        out[f"bits{k}"] = m.bits(r, words(n))
    lo, hi = m.bbox(g)
    out["bbox"] = np.concatenate([lo, hi])
    ids = [m.group_get_object(g, i) for i in range(n)]
    for o in removals:
        m.group_remove(g, int(o))
    for d in dirty:
        m.matrix_changed(g, int(d))
    if len(removals) or len(dirty):
        m.cull(g, r, vps[0])
        n2 = m.group_count(g)
        out["changed_after"] = m.changed(r).astype(np.int32)
        out["bits_after"] = m.bits(r, words(n2))
        out["order_after"] = np.array([m.group_get_object(g, i) for i in range(n2)], np.int32)
    out["ids"] = np.array(ids, np.int32)
    return out


def make_scenes(R):
    cases = {}
    # 1. plain configuration at reduced size (odd count: ragged last word and tile)
    sc = W.plain_scene(seed=10, n=4099)
    rng = np.random.default_rng(11)
    rem = rng.choice(4099, 40, replace=False)
    cases["plain4099"] = dict(lower=sc["lower"], upper=sc["upper"], xform=sc["xform"],
                              mats=sc["mats"], vps=sc["vps"], removals=rem)
    # 2. tiny sizes
    for n in (1, 31, 32, 33):
        s = W.plain_scene(seed=100 + n, n=n)
        s["lower"] *= 0  # boxes around the origin of each object
        cases[f"tiny{n}"] = dict(lower=s["lower"] - 1.0, upper=s["upper"] + 1.0, xform=s["xform"],
                                 mats=s["mats"] * np.float32(0.01), vps=s["vps"], removals=[0])
    # 3. camera inside the cloud: near-plane and behind-camera (w <= 0) cases
    rng = np.random.default_rng(12)
    n = 3000
    lower, upper, _ = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, n)
    mats[:, 12:15] *= np.float32(0.01)  # translations within +-10 of the camera
    P = W.perspective()
    vps = W.f32([W.look_at((0, 0, 0), (0, 0, -1), (0, 1, 0)) @ P, W.cube_face_views()[2],
                 W.cascade_views()[0]])
    cases["near_camera"] = dict(lower=lower, upper=upper, xform=np.arange(n, dtype=np.uint32),
                                mats=mats, vps=vps, removals=[])
    # 4. adversarial specials: NaN / inf / signed zero / subnormal / huge in boxes and matrices
    rng = np.random.default_rng(13)
    n = 2048
    lower = special_floats(rng, (3, n))
    upper = lower + np.abs(special_floats(rng, (3, n)))
    mats = special_floats(rng, (257, 16), 0.01)
    xform = rng.integers(0, 257, n, dtype=np.uint32)
    vps = np.concatenate([special_floats(rng, (2, 16), 0.0), W.f32([W.perspective()])])
    cases["specials"] = dict(lower=lower, upper=upper, xform=xform, mats=mats, vps=vps,
                             removals=[3, 2047, 1000], dirty=[0, 5])
    # 5. shared transforms: many objects per matrix, projective (non-affine) matrices
    rng = np.random.default_rng(14)
    n = 5000
    lower, upper, _ = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, 64)
    mats[::7, 3] = np.float32(0.001)  # non-zero w column
    mats[::5, 7] = np.float32(-0.0005)
    xform = rng.integers(0, 64, n, dtype=np.uint32)
    vps = W.f32(W.cube_face_views((10.0, -20.0, 5.0)) + W.stereo_views((0, 0, 50.0)))
    cases["shared_projective"] = dict(lower=lower, upper=upper, xform=xform, mats=mats, vps=vps,
                                      removals=[0, 4999])
    return cases


def make_tree(R):
    rng = np.random.default_rng(20)
    pairs, offsets, used = W.tree_levels(rng, 2500, depth=8)
    locs = W.random_matrices(rng, used)
    t = R.tree()
    for p, x in pairs:
        got = t.add(int(p), locs[x])
        assert got == x, (got, x)
    t.compute()
    out = dict(pairs=pairs, level_offsets=offsets, locals=locs, world0=t.world(used),
               dirty0=t.last_dirty()[: words(used)])
    upd = rng.choice(np.arange(1, used), 60, replace=False).astype(np.uint32)
    new = W.random_matrices(rng, 60)
    for k, i in enumerate(upd):
        t.update_local(int(i), new[k])
    t.compute()
    out.update(upd=upd, upd_locals=new, world1=t.world(used), dirty1=t.last_dirty()[: words(used)])
    # remove a level-2 transform (orphaning its level-3 children) and re-add a transform
    # that reuses its index under another level-2 parent: the new entry lands in level 3
    # after the orphans that still name it as parent, so within that level list the
    # readers precede the writer.  Recompute with every local dirty.
    victim = int(pairs[offsets[2] + 3][1])
    new_parent = int(pairs[offsets[2]][1])
    assert t.remove(victim) == 0
    reuse = t.add(new_parent, locs[victim])
    assert reuse == victim
    for i in range(1, used):
        t.update_local(i, locs[i])
    t.compute()
    out.update(victim=np.uint32(victim), world2=t.world(used), dirty2=t.last_dirty()[: words(used)])
    return out


def main():
    R = oracle.reference()
    if R is None:
        sys.exit("the reference sources are needed to write the golden fixtures")
    cases = make_scenes(R)
    for name, c in cases.items():
        res = scene_case(R, c["lower"], c["upper"], c["xform"], c["mats"], c["vps"],
                         c.get("removals", ()), c.get("dirty", ()))
        np.savez_compressed(OUT / f"scene_{name}.npz", lower=c["lower"], upper=c["upper"],
                            xform=c["xform"], mats=c["mats"], vps=c["vps"],
                            removals=np.asarray(c.get("removals", []), np.int32),
                            dirty=np.asarray(c.get("dirty", []), np.int32), **res)
    np.savez_compressed(OUT / "tree_small.npz", **make_tree(R))
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    main()
