"""Serving engine: every request's result is the same alone and in the mix (bit for bit),
and equals the oracle's cull; the mix is really batched, overlapped and evicting."""
import numpy as np
import pytest

import oracle
from pipeline_gb300 import native, serving
from pipeline_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_results_alone_equal_results_in_the_mix(ctx):
    templates = serving.make_templates(seed=5, n_templates=6, nmin=3_000, nmax=150_000)
    n_scenes = 18
    total = sum(serving.scene_bytes(templates[k % 6]["n"], templates[k % 6]["mats"].shape[0])
                for k in range(n_scenes))
    budget = int(total * 0.45)  # resident set smaller than the catalogue: eviction must run
    rng = np.random.default_rng(9)
    reqs = []
    for _ in range(60):
        scene = int(rng.integers(0, n_scenes))
        nv = int(rng.integers(1, 7))
        base = W.f32(W.cube_face_views(rng.uniform(-30, 30, 3)))[:nv]
        vps = np.stack([W.jitter_view(rng, v) for v in base])
        reqs.append((scene, vps))

    def run(mixed: bool):
        out = []
        with native.Server(ctx, budget, n_streams=3, max_batch_objects=4 << 20) as srv:
            for k in range(n_scenes):
                t = templates[k % 6]
                srv.add_scene(k, t["lower"], t["extent"], t["xform"], t["mats"])
            ids = []
            for scene, vps in reqs:
                ids.append(srv.submit(scene, vps, keep_bits=True))
                if not mixed:
                    srv.drain()
            srv.drain()
            comps = {c[0]: c for c in srv.poll()}
            for rid, (scene, vps) in zip(ids, reqs):
                t = templates[scene % 6]
                words = -(-t["n"] // 1024) * 32
                bits = [srv.result(rid, v, words)[: (t["n"] + 31) // 32] for v in range(len(vps))]
                out.append((bits, comps[rid][3]))
                srv.release(rid)
            stats = srv.stats()
        return out, stats

    alone, st_alone = run(False)
    mixed, st_mixed = run(True)
    assert st_mixed["scene_evictions"] > 0
    assert st_mixed["max_batch_requests"] > 1          # requests were batched together
    assert st_mixed["batches"] < st_alone["batches"]
    for (a_bits, a_vis), (m_bits, m_vis), (scene, vps) in zip(alone, mixed, reqs):
        assert a_vis == m_vis
        for a, m in zip(a_bits, m_bits):
            assert np.array_equal(a, m)
    # and the results are the reference cull's
    for (bits, vis), (scene, vps) in list(zip(mixed, reqs))[:12]:
        t = templates[scene % 6]
        for v, vp in enumerate(vps):
            exp = oracle.cull_bits(t["lower"], t["extent"], t["xform"], t["mats"], vp)
            assert np.array_equal(bits[v], exp)
            assert vis[v] == int(np.unpackbits(exp.view(np.uint8)).sum())


def test_submit_rejects_what_cannot_fit(ctx):
    t = serving.make_templates(seed=1, n_templates=1, nmin=50_000, nmax=50_001)[0]
    with native.Server(ctx, 1 << 20, n_streams=1) as srv:  # 1 MB budget, the scene needs ~1.8 MB
        srv.add_scene(0, t["lower"], t["extent"], t["xform"], t["mats"])
        with pytest.raises(native.DpcullError) as e:
            srv.submit(0, W.f32([W.perspective()]))
        assert e.value.code == native.ERR_CAPACITY


def test_scenes_added_while_serving(ctx):
    """Scenes with growing ids are registered from another thread while requests on the
    first scenes are admitted, launched and retired: the catalogue grows under the
    scheduler without disturbing it, and every result is still the oracle's."""
    import threading

    templates = serving.make_templates(seed=6, n_templates=3, nmin=2_000, nmax=40_000)
    rng = np.random.default_rng(10)
    reqs = []
    for _ in range(200):
        scene = int(rng.integers(0, 3))
        vps = W.f32(W.cube_face_views(rng.uniform(-20, 20, 3)))[: int(rng.integers(1, 7))]
        reqs.append((scene, vps))
    with native.Server(ctx, 1 << 30, n_streams=3, max_batch_objects=1 << 20) as srv:
        for k in range(3):
            t = templates[k]
            srv.add_scene(k, t["lower"], t["extent"], t["xform"], t["mats"])
        errors = []

        def add_more():
            try:
                for k in range(3, 3000):  # ids grow one by one: the scene table keeps growing
                    t = templates[k % 3]
                    srv.add_scene(k, t["lower"], t["extent"], t["xform"], t["mats"])
            except Exception as e:  # pragma: no cover - reported below
                errors.append(e)

        th = threading.Thread(target=add_more)
        th.start()
        ids, sent = [], []
        while th.is_alive() or len(ids) < len(reqs):  # requests flow while the table grows
            scene, vps = reqs[len(ids) % len(reqs)]
            keep = len(ids) % 7 == 0
            ids.append(srv.submit(scene, vps, keep_bits=keep))
            sent.append((scene, vps, keep))
        th.join()
        srv.drain()
        assert not errors
        comps = {c[0]: c for c in srv.poll()}
        assert len(comps) == len(ids)
        for rid, (scene, vps, keep) in zip(ids, sent):
            if not keep:
                continue
            t = templates[scene]
            words = -(-t["n"] // 1024) * 32
            for v, vp in enumerate(vps):
                got = srv.result(rid, v, words)[: (t["n"] + 31) // 32]
                assert np.array_equal(got, oracle.cull_bits(t["lower"], t["extent"], t["xform"], t["mats"], vp))

