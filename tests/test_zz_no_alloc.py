"""dpcull_cull_noalloc: the plain cull for callers that cannot allocate device memory
when they cull (a frame loop that must not hit cudaMalloc's implicit device
synchronisation, or a process whose device memory is all owned by another allocator).
It takes its scratch from a fixed static device array and the caller passes every input
and output buffer.  Two calls in a row must give the same visibility words and changed
lists as the regular entry point (dpcull_cull + its result), bit for bit.

The file name makes pytest collect it last, so that a run that stops at the first
failure (-x) has already run every other test if this one fails; the tests do not depend
on that order and pass alone in a fresh process too."""
import ctypes as C

import numpy as np
import pytest

import oracle
from pipeline_gb300 import native
from pipeline_gb300 import workloads as W

pytestmark = pytest.mark.gpu


class Buffers:
    """Caller-owned device buffers of one no-allocation cull (torch owns the memory)."""

    def __init__(self, lower, extent, xform, mats, cap):
        import torch

        n = len(xform)
        dev = torch.device("cuda", 0)
        rows = np.zeros((7, cap), np.float32)
        rows[0:3, :n] = lower
        rows[3:6, :n] = extent
        rows[6, :n] = np.ascontiguousarray(xform, np.uint32).view(np.float32)
        self.n, self.cap = n, cap
        self.objects = torch.from_numpy(rows).to(dev).contiguous()
        self.mats = torch.from_numpy(np.ascontiguousarray(mats, np.float32).reshape(-1, 16)).to(dev).contiguous()
        prev = np.zeros(cap // 32, np.uint32)  # a result that was never culled: all visible
        prev[: n // 32] = 0xFFFFFFFF
        if n % 32:
            prev[n // 32] = (1 << (n % 32)) - 1
        self.bits = torch.from_numpy(prev.view(np.int32)).to(dev)
        self.changed = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
        self.n_changed = torch.full((1,), 12345, dtype=torch.int32, device=dev)

    def cull(self, vp) -> int:
        import torch

        lib = native.load()
        v = np.ascontiguousarray(vp, np.float32).reshape(16)
        torch.cuda.synchronize()
        return lib.dpcull_cull_noalloc(C.c_void_p(self.objects.data_ptr()), self.cap, self.n,
                                       C.c_void_p(self.mats.data_ptr()), self.mats.shape[0], native.fptr(v),
                                       C.c_void_p(self.bits.data_ptr()), C.c_void_p(self.changed.data_ptr()),
                                       C.c_void_p(self.n_changed.data_ptr()), None)

    def result(self):
        k = int(self.n_changed.cpu().item())
        return (self.bits.cpu().numpy().view(np.uint32)[: (self.n + 31) // 32],
                self.changed.cpu().numpy().view(np.uint32)[:k])


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


def test_noalloc_at_its_maximum_size(ctx):
    """Exactly DPCULL_NOALLOC_MAX_OBJECTS objects (every delta word of the static scratch
    in use), two frames, against the regular entry point."""
    n = native.NOALLOC_MAX_OBJECTS
    rng = np.random.default_rng(32)
    lower, _, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, 8192)
    xform = rng.integers(0, 8192, n).astype(np.uint32)
    buf = Buffers(lower, extent, xform, mats, cap=n)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, mats)
    r = ctx.result_create(g)
    base = W.cube_face_views()[4]
    for vp in (base, W.jitter_view(rng, W.f32(base)[0], 10.0)):
        ctx.cull(g, r, vp)
        assert buf.cull(vp) == native.OK, native.load().dpcull_last_error().decode()
        bits, changed = buf.result()
        assert np.array_equal(bits, ctx.result_bits(r))
        assert np.array_equal(changed, ctx.result_changed(r))
        assert len(changed) > 0
    ctx.group_destroy(g)


def test_noalloc_empty_and_padded_and_bad_index(ctx):
    """n = 0 gives an empty changed list; a capacity past what n needs gives the same
    result as the regular entry point; a transform index past the matrix array is
    DPCULL_ERR_OUT_OF_RANGE with that object left invisible and every other object culled
    as usual."""
    rng = np.random.default_rng(33)
    vp = W.f32(W.cube_face_views()[0])[0]
    empty = Buffers(np.zeros((3, 0), np.float32), np.zeros((3, 0), np.float32), np.zeros(0, np.uint32),
                    W.random_matrices(rng, 1), cap=128)
    assert empty.cull(vp) == native.OK
    assert int(empty.n_changed.cpu().item()) == 0

    n = 5003
    lower, _, extent = W.random_boxes(rng, n)
    mats = W.random_matrices(rng, 256)
    mats[:, 12:15] *= np.float32(0.01)
    xform = rng.integers(0, 256, n).astype(np.uint32)
    padded = Buffers(lower, extent, xform, mats, cap=-(-n // 128) * 128 + 128)
    g = ctx.group_create()
    ctx.group_set_objects(g, lower, extent, xform)
    ctx.group_set_matrices(g, mats)
    r = ctx.result_create(g)
    ctx.cull(g, r, vp)
    assert padded.cull(vp) == native.OK
    bits, changed = padded.result()
    assert np.array_equal(bits, ctx.result_bits(r))
    assert np.array_equal(changed, ctx.result_changed(r))
    ctx.group_destroy(g)

    bad = 1234
    xf_bad = xform.copy()
    xf_bad[bad] = 256  # one past the matrix array
    buf = Buffers(lower, extent, xf_bad, mats, cap=-(-n // 128) * 128)
    assert buf.cull(vp) == native.ERR_OUT_OF_RANGE
    assert "transform index" in native.load().dpcull_last_error().decode()
    exp = oracle.cull_bits(lower, extent, xform, mats, vp)
    exp[bad >> 5] &= ~np.uint32(1 << (bad & 31))
    bits, changed = buf.result()
    assert np.array_equal(bits, exp)
    vis = np.unpackbits(exp.view(np.uint8), bitorder="little")[:n]
    assert np.array_equal(changed, np.flatnonzero(vis == 0))
