"""Multi-GPU host logic on CPU ranks (gloo, world size 2): object shards culled
independently and gathered equal the single-process cull (bits and changed lists)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from pipeline_gb300 import shard
from pipeline_gb300 import workloads as W


def free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def scene():
    sc = W.plain_scene(seed=21, n=10_001)
    vps = W.f32(W.cube_face_views()[:2])
    return sc, vps


def run_rank(rank, world, port, out):
    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, vps = scene()
    lo, ex, xf, first = shard.shard_objects(sc["lower"], sc["extent"], sc["xform"], world, rank)
    n = len(xf)
    prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
    if n % 32:
        prev[-1] = (1 << (n % 32)) - 1
    frames = []
    for vp in vps:
        bits = oracle.cull_bits(lo, ex, xf, sc["mats"], vp)  # stands in for the rank's GPU
        ch = oracle.update_changed(prev, bits, n)
        frames.append((bits, ch, n, first))
    gathered = [None] * world
    dist.all_gather_object(gathered, frames)
    if rank == 0:
        out.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_are_word_aligned():
    for n in (1, 31, 32, 33, 1000, 10_001):
        for w in (1, 2, 3, 8):
            spans = [shard.shard_bounds(n, w, r) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (b0, e0), (b1, e1) in zip(spans, spans[1:]):
                assert e0 == b1 and b1 % 32 == 0 or b1 == n


def test_two_cpu_ranks_equal_single_run():
    import oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=run_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    sc, vps = scene()
    n = len(sc["xform"])
    prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
    prev[-1] = (1 << (n % 32)) - 1
    for k, vp in enumerate(vps):
        bits = oracle.cull_bits(sc["lower"], sc["extent"], sc["xform"], sc["mats"], vp)
        ch = oracle.update_changed(prev, bits, n)
        parts = [g[k] for g in gathered]
        mb = shard.merge_bits([p[0] for p in parts], [p[2] for p in parts])
        mc = shard.merge_changed([p[1] for p in parts], [p[3] for p in parts])
        assert np.array_equal(mb, bits)
        assert np.array_equal(mc, ch)


def run_rank_gather(rank, world, port, out):
    """One CPU rank of a sharded step: cull its shard (the oracle stands in for the rank's
    GPU) and gather through shard.gather_results, the code bench.py's multi-GPU end-to-end
    leg runs."""
    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, vps = scene()
    lo, ex, xf, first = shard.shard_objects(sc["lower"], sc["extent"], sc["xform"], world, rank)
    n = len(xf)
    bits, changed, counts = [], [], []
    for vp in vps:  # one new result per view: each starts all visible
        prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
        if n % 32:
            prev[-1] = (1 << (n % 32)) - 1
        b = oracle.cull_bits(lo, ex, xf, sc["mats"], vp)
        ch = oracle.update_changed(prev, b, n)
        bits.append(b)
        buf = np.zeros(n + 5, np.uint32)  # list buffers are longer than the lists
        buf[: len(ch)] = ch
        changed.append(buf)
        counts.append(len(ch))
    res = shard.gather_results(bits, changed, counts, n, first)
    if rank == 0:
        out.put(res)
    else:
        assert res is None
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gather_results_over_cpu_ranks(world):
    import oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=run_rank_gather, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    merged_bits, merged_changed = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    sc, vps = scene()
    n = len(sc["xform"])
    for k, vp in enumerate(vps):
        prev = np.full((n + 31) // 32, 0xFFFFFFFF, np.uint32)
        prev[-1] = (1 << (n % 32)) - 1
        bits = oracle.cull_bits(sc["lower"], sc["extent"], sc["xform"], sc["mats"], vp)
        ch = oracle.update_changed(prev, bits, n)
        assert np.array_equal(merged_bits[k], bits)
        assert np.array_equal(merged_changed[k], ch)
