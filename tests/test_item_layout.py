"""The cull's work-item layout (pipeline_gb300/csrc/dpcull_internal.h), compiled for the
host: item_tiles-tile items, then single-tile items for the launch's last `tail` units.
Every tile of every scene is covered exactly once, items are numbered scene after scene,
and the launch ends with at least min(tail, all units) single-tile units."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "item_layout.cpp"


def cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("layout") / "liblayout.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I", str(ROOT / "pipeline_gb300" / "csrc"),
                    "-I", cuda_include(), str(SRC), "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
    L.layout_items.restype = C.c_uint32
    L.layout_items.argtypes = [C.c_size_t, u32p, u32p, C.c_uint32, C.c_uint64, u32p, u32p]
    L.groups_of.restype = C.c_uint32
    L.groups_of.argtypes = [C.c_uint32] * 3
    L.tiles_for.restype = C.c_uint32
    L.tiles_for.argtypes = [C.c_uint64, C.c_int]
    L.tail_for.restype = C.c_uint64
    L.tail_for.argtypes = [C.c_int]
    return L


def tiles_of_group(g, n_tiles, n_big, it):
    """The kernel's mapping (cull.cu warp_item): big groups first, then one tile each."""
    if g < n_big:
        first = g * it
        return list(range(first, min(first + it, n_tiles)))
    return [n_big * it + (g - n_big)]


def check(lib, tiles, vgroups, it, tail):
    n = len(tiles)
    t = np.asarray(tiles, np.uint32)
    vg = np.asarray(vgroups, np.uint32)
    n_big = np.zeros(n, np.uint32)
    begin = np.zeros(n, np.uint32)
    items = lib.layout_items(n, t, vg, it, tail, n_big, begin)
    expect_begin = 0
    singles_at_end = []
    for i in range(n):
        assert begin[i] == expect_begin
        groups = lib.groups_of(int(t[i]), int(n_big[i]), it)
        covered = np.zeros(int(t[i]), np.int64)
        sizes = []
        for g in range(groups):
            ts = tiles_of_group(g, int(t[i]), int(n_big[i]), it)
            assert ts and all(0 <= x < t[i] for x in ts)
            covered[ts] += 1
            sizes.append(len(ts))
        assert (covered == 1).all(), (i, tiles[i], n_big[i])
        if n_big[i] * it < t[i]:  # single-tile groups sit after the big ones
            assert all(s == 1 for s in sizes[int(n_big[i]):])
        expect_begin += groups * int(vg[i])
        singles_at_end.append(sizes)
    assert items == expect_begin
    # the launch's last units: at least min(tail, all units) of them are single tiles
    if it > 1 and tail:
        units = 0
        for i in reversed(range(n)):
            for s in reversed(singles_at_end[i]):
                if s != 1:
                    break
                units += int(vg[i])
            else:
                continue
            break
        total = int(sum(int(a) * int(b) for a, b in zip(tiles, vgroups)))
        assert units >= min(tail, total) or units == total
    return n_big, items


def test_layout_random_scene_lists(lib):
    rng = np.random.default_rng(5)
    for _ in range(300):
        n = int(rng.integers(1, 12))
        tiles = rng.integers(0, 3000, n).tolist()
        vgroups = rng.integers(1, 4, n).tolist()
        it = int(rng.choice([1, 2, 4]))
        tail = int(rng.choice([0, 1, 7, 64, 500, 9728]))
        check(lib, tiles, vgroups, it, tail)


def test_layout_stress_workload(lib):
    """16M objects, one view group, 152 SMs: 8-tile items and a 9728-unit single-tile tail."""
    tiles = 16_000_000 // 128
    it = lib.tiles_for(tiles, 152)
    tail = lib.tail_for(152)
    assert it == 8 and tail == 152 * 64
    n_big, items = check(lib, [tiles], [1], it, tail)
    assert n_big[0] == (tiles - tail) // 8
    assert items == n_big[0] + (tiles - n_big[0] * 8)


def test_layout_without_tail_keeps_full_items(lib):
    n_big, items = check(lib, [10, 0, 7], [2, 3, 1], 4, 0)
    assert n_big.tolist() == [3, 0, 2] and items == 3 * 2 + 0 + 2
    n_big, _ = check(lib, [10], [1], 1, 50)  # one tile per item already
    assert n_big.tolist() == [10]
