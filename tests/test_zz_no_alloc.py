"""dpcull_cull_noalloc: the plain cull for callers that cannot allocate device memory
when they cull (a frame loop that must not hit cudaMalloc's implicit device
synchronisation, or a process whose device memory is all owned by another allocator).
It takes its scratch from a fixed static device array and the caller passes every input
and output buffer.  Two calls in a row must give the same visibility words and changed
lists as the regular entry point (dpcull_cull + its result), bit for bit.

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from pipeline_gb300 import native
from pipeline_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point_twice(ctx):
    import torch

    lib = native.load()
    sc = W.plain_scene(seed=31, n=70_001)
    n = len(sc["xform"])
    cap = -(-n // 1024) * 1024
    dev = torch.device("cuda", 0)
    rows = np.zeros((7, cap), np.float32)
    rows[0:3, :n] = sc["lower"]
    rows[3:6, :n] = sc["extent"]
    rows[6, :n] = sc["xform"].view(np.float32)
    objects = torch.from_numpy(rows).to(dev).contiguous()
    mats = torch.from_numpy(sc["mats"]).to(dev).contiguous()
    words = cap // 32
    prev = np.zeros(words, np.uint32)  # a new result starts all visible
    prev[: n // 32] = 0xFFFFFFFF
    if n % 32:
        prev[n // 32] = (1 << (n % 32)) - 1
    bits = torch.from_numpy(prev.view(np.int32)).to(dev)
    changed = torch.zeros(n, dtype=torch.int32, device=dev)
    n_changed = torch.zeros(1, dtype=torch.int32, device=dev)

    g = ctx.group_create()
    ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
    ctx.group_set_matrices(g, sc["mats"])
    r = ctx.result_create(g)

    vps = [sc["vps"][0], sc["vps"][1]]
    for vp in vps:
        ctx.cull(g, r, vp)
        exp_bits = ctx.result_bits(r)
        exp_changed = ctx.result_changed(r)
        v = np.ascontiguousarray(vp, np.float32).reshape(16)
        torch.cuda.synchronize()
        rc = lib.dpcull_cull_noalloc(C.c_void_p(objects.data_ptr()), cap, n, C.c_void_p(mats.data_ptr()),
                                     mats.shape[0], native.fptr(v), C.c_void_p(bits.data_ptr()),
                                     C.c_void_p(changed.data_ptr()), C.c_void_p(n_changed.data_ptr()), None)
        assert rc == native.OK, lib.dpcull_last_error().decode()
        got_bits = bits.cpu().numpy().view(np.uint32)[: (n + 31) // 32]
        k = int(n_changed.cpu().item())
        got_changed = changed.cpu().numpy().view(np.uint32)[:k]
        assert np.array_equal(got_bits, exp_bits)
        assert np.array_equal(got_changed, exp_changed)
    ctx.group_destroy(g)


def test_noalloc_rejects_sizes_past_its_maximum():
    lib = native.load()
    too_many = native.NOALLOC_MAX_OBJECTS + 1
    cap = -(-too_many // 1024) * 1024
    v = np.eye(4, dtype=np.float32).reshape(16)
    rc = lib.dpcull_cull_noalloc(None, cap, too_many, None, 1, native.fptr(v), None, None, None, None)
    assert rc == native.ERR_CAPACITY
    assert "DPCULL_NOALLOC_MAX_OBJECTS" in lib.dpcull_last_error().decode()
