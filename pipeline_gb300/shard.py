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
