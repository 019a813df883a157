"""Object sharding across GPUs (one process per GPU).

Each object's visibility depends only on its own box, its world matrix and the view, so
a group splits into contiguous object ranges with no exchange on the data path.  Ranges
start on multiples of 32 objects, so no visibility word is split: the shards' words
concatenate into the whole group's words, and the shards' changed lists (shard-local
ascending indices plus the shard's first object) concatenate, in rank order, into the
whole group's ascending changed list.  World matrices are replicated (each shard needs
the ones its objects reference).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n_objects: int, world: int, rank: int) -> tuple[int, int]:
    """[begin, end) of the objects of `rank`; begin is a multiple of 32."""
    per = -(-n_objects // (32 * world)) * 32
    b = min(n_objects, rank * per)
    return b, min(n_objects, b + per)


def shard_objects(lower, extent, xform, world: int, rank: int):
    b, e = shard_bounds(len(xform), world, rank)
    return lower[:, b:e], extent[:, b:e], xform[b:e], b


def merge_bits(parts: list[np.ndarray], counts: list[int]) -> np.ndarray:
    """Concatenates the shards' visibility words (each shard's count is a multiple of 32
    except possibly the last one)."""
    out = []
    for p, c in zip(parts, counts):
        out.append(np.asarray(p, np.uint32)[: (c + 31) // 32])
    return np.concatenate(out) if out else np.zeros(0, np.uint32)


def merge_changed(parts: list[np.ndarray], firsts: list[int]) -> np.ndarray:
    """Concatenates shard-local ascending changed lists into the group's list."""
    out = [np.asarray(p, np.uint32) + np.uint32(f) for p, f in zip(parts, firsts)]
    return np.concatenate(out) if out else np.zeros(0, np.uint32)


def gather_results(bits: list, changed: list, n_changed, count: int, first: int, group=None, dst: int = 0):
    """Gathers every rank's results of one step to rank `dst` and merges them into the
    whole group's: per view, the visibility words (the rank's `count` objects from global
    object `first` on) and the first n_changed[v] entries of its shard-local changed list.
    Host tensors over torch.distributed (a gloo group beside NCCL works).  Returns
    (words per view, changed list per view) on `dst`, None elsewhere."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    n_views = len(bits)
    meta = torch.tensor([count, first, *[int(x) for x in n_changed]], dtype=torch.int64)
    metas = [torch.zeros_like(meta) for _ in range(world)]
    dist.all_gather(metas, meta, group=group)
    sizes = [sum((int(m[0]) + 31) // 32 for _ in range(n_views)) + int(m[2:].sum()) for m in metas]
    cap = max(sizes)
    words = (count + 31) // 32
    parts = [np.asarray(b, np.uint32)[:words] for b in bits]
    parts += [np.asarray(c, np.uint32)[: int(k)] for c, k in zip(changed, n_changed)]
    buf = np.zeros(cap, np.uint32)
    flat = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
    buf[: flat.size] = flat
    t = torch.from_numpy(buf.view(np.int32))
    out = [torch.zeros(cap, dtype=torch.int32) for _ in range(world)] if rank == dst else None
    dist.gather(t, out, dst=dst, group=group)
    if rank != dst:
        return None
    merged_bits, merged_changed = [], []
    per_rank = []
    for m, tr in zip(metas, out):
        a = tr.numpy().view(np.uint32)
        c, w = int(m[0]), (int(m[0]) + 31) // 32
        ks = [int(x) for x in m[2:]]
        off = 0
        bl = []
        for _ in range(n_views):
            bl.append(a[off:off + w])
            off += w
        cl = []
        for k in ks:
            cl.append(a[off:off + k])
            off += k
        per_rank.append((c, int(m[1]), bl, cl))
    for v in range(n_views):
        merged_bits.append(merge_bits([p[2][v] for p in per_rank], [p[0] for p in per_rank]))
        merged_changed.append(merge_changed([p[3][v] for p in per_rank], [p[1] for p in per_rank]))
    return merged_bits, merged_changed
