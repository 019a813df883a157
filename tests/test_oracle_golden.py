"""The C restatement (oracle port) against golden fixtures written by the reference itself."""
import numpy as np
import pytest

from conftest import f32_bits, golden_scene_names, load_golden


def replay_scene(m, z):
    """Replays the fixture's operation sequence on a Manager (port or reference)."""
    g = m.group()
    r = m.result(g)
    n = len(z["xform"])
    m.add_boxes(g, z["lower"], z["upper"], z["xform"])
    m.set_matrices(g, z["mats"])
    out = {}
    for k, vp in enumerate(z["vps"]):
        m.cull(g, r, vp)
        out[f"changed{k}"] = m.changed(r)
        out[f"bits{k}"] = m.bits(r, (n + 31) // 32)
    lo, hi = m.bbox(g)
    out["bbox"] = np.concatenate([lo, hi])
    for o in z["removals"]:
        assert m.group_remove(g, int(o)) == 0
    for d in z["dirty"]:
        m.matrix_changed(g, int(d))
    if len(z["removals"]) or len(z["dirty"]):
        m.cull(g, r, z["vps"][0])
        n2 = m.group_count(g)
        out["changed_after"] = m.changed(r)
        out["bits_after"] = m.bits(r, (n2 + 31) // 32)
        out["order_after"] = np.array([m.group_get_object(g, i) for i in range(n2)], np.int32)
    return out


@pytest.mark.parametrize("name", golden_scene_names())
def test_port_matches_golden_scene(port, name):
    z = load_golden(name)
    out = replay_scene(port.manager(), z)
    for k, v in out.items():
        if k == "bbox":
            assert np.array_equal(f32_bits(v), f32_bits(z[k])), name
        else:
            assert np.array_equal(np.asarray(v), z[k]), (name, k)


def test_port_matches_golden_tree(port):
    z = load_golden("tree_small.npz")
    pairs, locs = z["pairs"], z["locals"]
    used = locs.shape[0]
    words = (used + 31) // 32
    t = port.tree()
    for p, x in pairs:
        assert t.add(int(p), locs[x]) == x
    t.compute()
    assert np.array_equal(f32_bits(t.world(used)), f32_bits(z["world0"]))
    assert np.array_equal(t.last_dirty()[:words], z["dirty0"])
    for k, i in enumerate(z["upd"]):
        t.update_local(int(i), z["upd_locals"][k])
    t.compute()
    assert np.array_equal(f32_bits(t.world(used)), f32_bits(z["world1"]))
    assert np.array_equal(t.last_dirty()[:words], z["dirty1"])
    victim = int(z["victim"])
    offs = z["level_offsets"]
    new_parent = int(pairs[offs[2]][1])
    assert t.remove(victim) == 0
    assert t.add(new_parent, locs[victim]) == victim
    for i in range(1, used):
        t.update_local(i, locs[i])
    t.compute()
    assert np.array_equal(f32_bits(t.world(used)), f32_bits(z["world2"]))
    assert np.array_equal(t.last_dirty()[:words], z["dirty2"])


def test_first_cull_semantics(port):
    """ResultBitSet starts all-visible: the first changed list is the invisible objects."""
    z = load_golden("scene_plain4099.npz")
    n = len(z["xform"])
    bits = z["bits0"]
    vis = np.unpackbits(bits.view(np.uint8), bitorder="little")[:n].astype(bool)
    assert np.array_equal(z["changed0"], np.nonzero(~vis)[0])


def test_changed_is_xor_of_frames(port):
    z = load_golden("scene_plain4099.npz")
    n = len(z["xform"])
    v0 = np.unpackbits(z["bits0"].view(np.uint8), bitorder="little")[:n]
    v1 = np.unpackbits(z["bits1"].view(np.uint8), bitorder="little")[:n]
    assert np.array_equal(z["changed1"], np.nonzero(v0 ^ v1)[0])


def test_math_kernels_order(port):
    """Vec4*Mat44 and Mat44*Mat44 use the left-to-right 4-term sums of Matmnt.h:1371-1415."""
    import oracle

    rng = np.random.default_rng(0)
    for _ in range(200):
        v = rng.standard_normal(4).astype(np.float32) * np.float32(1e3)
        m = rng.standard_normal(16).astype(np.float32)
        M = m.reshape(4, 4)
        exp = np.zeros(4, np.float32)
        for j in range(4):
            acc = np.float32(v[0] * M[0, j])
            acc = np.float32(acc + np.float32(v[1] * M[1, j]))
            acc = np.float32(acc + np.float32(v[2] * M[2, j]))
            acc = np.float32(acc + np.float32(v[3] * M[3, j]))
            exp[j] = acc
        assert np.array_equal(f32_bits(oracle.vec4_mul_mat44(v, m)), f32_bits(exp))
        b = rng.standard_normal(16).astype(np.float32)
        got = oracle.mat44_mul(m, b).reshape(4, 4)
        for i in range(4):
            assert np.array_equal(f32_bits(got[i]), f32_bits(oracle.vec4_mul_mat44(M[i], b)))
