"""dp::transform::Tree on the GPU.

Host side: the tree's structure exactly as the reference keeps it
(dp/transform/Tree.h:42-129, src/Tree.cpp): indices allocated first-free from a free bit
array grown in steps of 65536, a level per transform (root 0 at level -1), and per-level
lists of (parent, transform) entries in insertion order with swap-with-last removal.
Device side (libdpcull): local / world matrices, dirty bits and the level-ordered
propagation kernel.  compute() uploads the structure when it changed and the local
matrices set since the last compute, then propagates on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import native

VECTOR_GROWTH = 65536  # Tree.cpp:35


class Tree:
    def __init__(self, ctx: native.Context, capacity: int = VECTOR_GROWTH):
        self.ctx = ctx
        self.capacity = int(capacity)
        self.handle = ctx.tree_create(self.capacity)
        self._free = np.ones(self.capacity, bool)
        self._free[0] = False
        self._level = np.zeros(self.capacity, np.uint32)
        self._level[0] = 0xFFFFFFFF
        self._levels: list[list[tuple[int, int]]] = []
        self._pending: dict[int, np.ndarray] = {}
        self._structure_dirty = True

    # ---- structure (host) ---------------------------------------------------------------
    def _valid(self, i: int) -> bool:
        return 0 <= i < self.capacity and not self._free[i]

    def _grow(self) -> None:
        """Tree::resizeDataStructures (Tree.cpp:117-126): device arrays keep their contents."""
        new_cap = self.capacity + VECTOR_GROWTH
        self.ctx.tree_resize(self.handle, new_cap)
        self._free = np.concatenate([self._free, np.ones(VECTOR_GROWTH, bool)])
        self._level = np.concatenate([self._level, np.zeros(VECTOR_GROWTH, np.uint32)])
        self.capacity = new_cap
        self._structure_dirty = True

    def add_transform(self, parent: int, matrix) -> int:
        """Tree::addTransform (Tree.cpp:54-76)."""
        if not self._valid(parent):
            raise RuntimeError("Tree::addTransform: Parent does not exist")
        free = np.flatnonzero(self._free)
        if free.size == 0:
            self._grow()
            free = np.flatnonzero(self._free)
        idx = int(free[0])
        self._free[idx] = False
        lvl = (int(self._level[parent]) + 1) & 0xFFFFFFFF
        self._level[idx] = lvl
        while len(self._levels) <= lvl:
            self._levels.append([])
        self._levels[lvl].append((int(parent), idx))
        self._pending[idx] = np.asarray(matrix, np.float32).reshape(16).copy()
        self._structure_dirty = True
        return idx

    def remove_transform(self, index: int) -> None:
        """Tree::removeTransform (Tree.cpp:78-98): children are left orphaned."""
        if not self._valid(index):
            raise RuntimeError("Tree::removeTransform: Transform does not exist")
        lst = self._levels[int(self._level[index])]
        for e, (_, t) in enumerate(lst):
            if t == index:
                lst[e] = lst[-1]
                lst.pop()
                break
        self._free[index] = True
        self._pending.pop(index, None)
        self._structure_dirty = True

    def update_local_matrix(self, index: int, matrix) -> None:
        """Tree::updateLocalMatrix (Tree.h:87)."""
        self._pending[int(index)] = np.asarray(matrix, np.float32).reshape(16).copy()

    def level_lists(self):
        pairs = [p for lvl in self._levels for p in lvl]
        offsets = np.cumsum([0] + [len(l) for l in self._levels]).astype(np.uint32)
        return np.asarray(pairs, np.uint32).reshape(-1, 2), offsets

    # ---- device ------------------------------------------------------------------------
    def compute(self) -> None:
        """Tree::compute (Tree.cpp:133-166) on the GPU (asynchronous)."""
        if self._structure_dirty:
            pairs, offsets = self.level_lists()
            self.ctx.tree_set_structure(self.handle, pairs, offsets)
            self._structure_dirty = False
        if self._pending:
            idx = np.fromiter(self._pending.keys(), np.uint32, len(self._pending))
            mats = np.stack(list(self._pending.values()))
            self.ctx.tree_set_locals(self.handle, idx, mats)
            self._pending.clear()
        self.ctx.tree_compute(self.handle)

    def get_transform_count(self) -> int:
        return self.capacity

    def world_matrices(self, count: int | None = None) -> np.ndarray:
        return self.ctx.tree_world(self.handle, 0, self.capacity if count is None else count)

    def world_device(self):
        return self.ctx.tree_world_device(self.handle)

    def dirty_world_matrices(self) -> np.ndarray:
        return self.ctx.tree_dirty_world(self.handle, (self.capacity + 31) // 32)
