"""ctypes binding of the C ABI in include/dpcull.h (libdpcull.so).

This is the product path from Python: every call goes to the CUDA library.  There is
no CPU fallback; if the library or a GPU is missing the calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libdpcull.so"

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_OUT_OF_RANGE = -2
ERR_CUDA = -3
ERR_NO_MEMORY = -4
ERR_STATE = -5
ERR_TIMEOUT = -6
ERR_CAPACITY = -7

_P = C.c_void_p
_U32 = C.c_uint32
_SZ = C.c_size_t
_I = C.c_int
_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)


class DpcullError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dpcull error {code}: {msg}")
        self.code = code


class Job(C.Structure):
    _fields_ = [("group", _U32), ("n_views", _U32), ("results", _UP), ("vps", _FP)]


class Tuning(C.Structure):
    _fields_ = [("views_per_pass", _U32), ("tiles_per_ticket", _U32), ("ctas_per_sm", _U32),
                ("reserved", _U32)]

    def as_dict(self) -> dict:
        return {"views_per_pass": self.views_per_pass, "tiles_per_ticket": self.tiles_per_ticket,
                "ctas_per_sm": self.ctas_per_sm}


_SIGS = {
    "dpcull_last_error": (C.c_char_p, []),
    "dpcull_version": (_U32, []),
    "dpcull_ctx_create": (_I, [_I, _P, C.POINTER(_P)]),
    "dpcull_ctx_destroy": (_I, [_P]),
    "dpcull_ctx_synchronize": (_I, [_P]),
    "dpcull_ctx_stream": (_P, [_P]),
    "dpcull_ctx_kernel_launches": (C.c_uint64, [_P]),
    "dpcull_ctx_device_bytes": (C.c_uint64, [_P]),
    "dpcull_ctx_set_prefilter": (_I, [_P, _I]),
    "dpcull_ctx_set_box_cache": (_I, [_P, _I]),
    "dpcull_ctx_cull_launches": (_I, [_P, C.POINTER(C.c_uint64)]),
    "dpcull_group_create": (_I, [_P, _UP]),
    "dpcull_group_destroy": (_I, [_P, _U32]),
    "dpcull_group_set_objects": (_I, [_P, _U32, _SZ, _FP, _FP, _UP]),
    "dpcull_group_append_objects": (_I, [_P, _U32, _SZ, _FP, _FP, _UP]),
    "dpcull_group_update_objects": (_I, [_P, _U32, _SZ, _UP, _FP, _FP, _UP]),
    "dpcull_group_remove_object": (_I, [_P, _U32, _SZ]),
    "dpcull_group_count": (_I, [_P, _U32, C.POINTER(_SZ)]),
    "dpcull_group_set_matrices": (_I, [_P, _U32, _P, _SZ, _SZ]),
    "dpcull_group_update_matrices": (_I, [_P, _U32, _SZ, _UP, _P, _SZ]),
    "dpcull_group_bind_device_matrices": (_I, [_P, _U32, _P, _SZ]),
    "dpcull_group_bounding_box": (_I, [_P, _U32, _FP, _FP]),
    "dpcull_result_create": (_I, [_P, _U32, _UP]),
    "dpcull_result_destroy": (_I, [_P, _U32]),
    "dpcull_cull": (_I, [_P, _U32, _U32, _FP]),
    "dpcull_result_changed": (_I, [_P, _U32, _UP, _SZ, C.POINTER(_SZ)]),
    "dpcull_result_bits": (_I, [_P, _U32, _UP, _SZ, C.POINTER(_SZ)]),
    "dpcull_result_read": (_I, [_P, _U32, C.c_void_p, _SZ, C.c_void_p, C.c_void_p, _SZ, C.c_void_p]),
    "dpcull_result_is_visible": (_I, [_P, _U32, _SZ, C.POINTER(_I)]),
    "dpcull_result_device": (_I, [_P, _U32, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "dpcull_result_move": (_I, [_P, _U32, _SZ, _SZ]),
    "dpcull_cull_batched": (_I, [_P, C.POINTER(Job), _SZ, C.POINTER(Tuning)]),
    "dpcull_plan_create": (_I, [_P, C.POINTER(Job), _SZ, C.POINTER(Tuning), _UP]),
    "dpcull_plan_set_views": (_I, [_P, _U32, _FP]),
    "dpcull_plan_launch": (_I, [_P, _U32]),
    "dpcull_plan_tuning": (_I, [_P, _U32, C.POINTER(Tuning)]),
    "dpcull_plan_kernel_ms": (_I, [_P, _U32, _U32, C.POINTER(C.c_float)]),
    "dpcull_plan_read": (_I, [_P, _U32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "dpcull_plan_read_async": (_I, [_P, _U32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "dpcull_plan_read_wait": (_I, [_P, _U32]),
    "dpcull_plan_snapshot": (_I, [_P, _U32]),
    "dpcull_plan_destroy": (_I, [_P, _U32]),
    "dpcull_autotune": (_I, [_P, C.POINTER(Job), _SZ, C.POINTER(Tuning)]),
    "dpcull_tree_create": (_I, [_P, _SZ, _UP]),
    "dpcull_tree_destroy": (_I, [_P, _U32]),
    "dpcull_tree_resize": (_I, [_P, _U32, _SZ]),
    "dpcull_tree_set_structure": (_I, [_P, _U32, _SZ, _UP, _SZ, _UP]),
    "dpcull_tree_set_locals": (_I, [_P, _U32, _SZ, _UP, _FP]),
    "dpcull_tree_set_worlds": (_I, [_P, _U32, _SZ, _UP, _FP]),
    "dpcull_tree_compute": (_I, [_P, _U32]),
    "dpcull_tree_world_device": (_I, [_P, _U32, C.POINTER(_P), C.POINTER(_SZ)]),
    "dpcull_tree_world": (_I, [_P, _U32, _SZ, _SZ, _FP]),
    "dpcull_tree_dirty_world": (_I, [_P, _U32, _UP, _SZ]),
    "dpcull_cull_noalloc": (_I, [_P, _SZ, _SZ, _P, _SZ, _FP, _P, _P, _P, _P]),
    "dpcull_server_now": (C.c_double, []),
    "dpcull_server_create": (_I, [_P, C.c_uint64, _U32, C.c_uint64, C.POINTER(_P)]),
    "dpcull_server_destroy": (_I, [_P]),
    "dpcull_server_add_scene": (_I, [_P, _U32, _SZ, _FP, _FP, _UP, _FP, _SZ]),
    "dpcull_server_submit": (_I, [_P, _U32, _U32, _FP, _U32, C.POINTER(C.c_uint64)]),
    "dpcull_server_poll": (_I, [_P, _P, _SZ, C.POINTER(_SZ)]),
    "dpcull_server_result": (_I, [_P, C.c_uint64, _U32, _UP, _SZ]),
    "dpcull_server_release": (_I, [_P, C.c_uint64]),
    "dpcull_server_drain": (_I, [_P]),
    "dpcull_server_get_stats": (_I, [_P, _P]),
}

SERVER_MAX_VIEWS = 8
REQUEST_KEEP_BITS = 1


class Completion(C.Structure):
    _fields_ = [("request", C.c_uint64), ("scene", _U32), ("n_views", _U32),
                ("visible", _U32 * SERVER_MAX_VIEWS), ("objects", C.c_uint64),
                ("submit_s", C.c_double), ("start_s", C.c_double), ("done_s", C.c_double),
                ("status", C.c_int32), ("pad", _U32)]


class ServerStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "requests_submitted", "requests_completed", "batches", "scene_uploads", "scene_evictions",
        "upload_bytes", "resident_bytes", "resident_scenes", "budget_bytes", "max_batch_requests",
        "pending_requests", "max_turn_us", "slow_turns", "max_upload_call_us", "max_evict_call_us",
        "reserved_bytes")]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}

NOALLOC_MAX_OBJECTS = 1 << 20  # DPCULL_NOALLOC_MAX_OBJECTS

_lib = None


def load() -> C.CDLL:
    """Loads libdpcull.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run pipeline_gb300.build.build_all() first "
                               "(the culling backend has no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(rc: int) -> None:
    if rc != OK:
        raise DpcullError(rc, load().dpcull_last_error().decode())


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def uptr(a: np.ndarray):
    return a.ctypes.data_as(_UP)


class Context:
    """One dpcull context (one CUDA stream) on one device."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        h = _P()
        _check(self.lib.dpcull_ctx_create(device, stream, C.byref(h)))
        self.h = h
        self._keep: dict = {}

    def close(self) -> None:
        if self.h:
            _check(self.lib.dpcull_ctx_destroy(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- context ----
    def synchronize(self) -> None:
        _check(self.lib.dpcull_ctx_synchronize(self.h))

    @property
    def stream(self) -> int:
        return self.lib.dpcull_ctx_stream(self.h) or 0

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.dpcull_ctx_kernel_launches(self.h))

    def cull_launches(self) -> dict:
        """Cull-kernel launches so far by kind: fused (no box cache), fill (stores it), read."""
        out = (C.c_uint64 * 3)()
        _check(self.lib.dpcull_ctx_cull_launches(self.h, out))
        return {"fused": int(out[0]), "fill": int(out[1]), "read": int(out[2])}

    @property
    def device_bytes(self) -> int:
        return int(self.lib.dpcull_ctx_device_bytes(self.h))

    def set_prefilter(self, enabled: bool) -> None:
        _check(self.lib.dpcull_ctx_set_prefilter(self.h, 1 if enabled else 0))

    def set_box_cache(self, enabled: bool) -> None:
        """Keep (default) or recompute the groups' boxes between culls (identical results)."""
        _check(self.lib.dpcull_ctx_set_box_cache(self.h, 1 if enabled else 0))

    # ---- groups ----
    def group_create(self) -> int:
        g = _U32()
        _check(self.lib.dpcull_group_create(self.h, C.byref(g)))
        return g.value

    def group_destroy(self, g: int) -> None:
        _check(self.lib.dpcull_group_destroy(self.h, g))

    def group_set_objects(self, g: int, lower, extent, xform) -> None:
        lo, ex, xf = _f32(lower), _f32(extent), _u32(xform)
        n = xf.shape[0]
        assert lo.shape == (3, n) and ex.shape == (3, n)
        _check(self.lib.dpcull_group_set_objects(self.h, g, n, fptr(lo), fptr(ex), uptr(xf)))

    def group_append_objects(self, g: int, lower, extent, xform) -> None:
        lo, ex, xf = _f32(lower), _f32(extent), _u32(xform)
        _check(self.lib.dpcull_group_append_objects(self.h, g, xf.shape[0], fptr(lo), fptr(ex), uptr(xf)))

    def group_update_objects(self, g: int, index, lower, extent, xform) -> None:
        ix, lo, ex, xf = _u32(index), _f32(lower), _f32(extent), _u32(xform)
        _check(self.lib.dpcull_group_update_objects(self.h, g, ix.shape[0], uptr(ix), fptr(lo), fptr(ex), uptr(xf)))

    def group_remove_object(self, g: int, index: int) -> None:
        _check(self.lib.dpcull_group_remove_object(self.h, g, index))

    def group_count(self, g: int) -> int:
        n = _SZ()
        _check(self.lib.dpcull_group_count(self.h, g, C.byref(n)))
        return n.value

    def group_set_matrices(self, g: int, mats: np.ndarray, stride: int | None = None) -> None:
        m = np.ascontiguousarray(mats)
        count = m.shape[0]
        st = stride if stride is not None else (m.strides[0] if count else 64)
        _check(self.lib.dpcull_group_set_matrices(self.h, g, m.ctypes.data if count else None, count, st))

    def group_update_matrices(self, g: int, index, mats: np.ndarray, stride: int | None = None) -> None:
        ix = _u32(index)
        m = np.ascontiguousarray(mats)
        st = stride if stride is not None else m.strides[0]
        _check(self.lib.dpcull_group_update_matrices(self.h, g, ix.shape[0], uptr(ix), m.ctypes.data, st))

    def group_bind_device_matrices(self, g: int, dev_ptr: int, count: int) -> None:
        _check(self.lib.dpcull_group_bind_device_matrices(self.h, g, dev_ptr, count))

    def group_bounding_box(self, g: int):
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        _check(self.lib.dpcull_group_bounding_box(self.h, g, fptr(lo), fptr(hi)))
        return lo, hi

    # ---- results ----
    def result_create(self, g: int) -> int:
        r = _U32()
        _check(self.lib.dpcull_result_create(self.h, g, C.byref(r)))
        return r.value

    def result_destroy(self, r: int) -> None:
        _check(self.lib.dpcull_result_destroy(self.h, r))

    def cull(self, g: int, r: int, vp) -> None:
        v = _f32(vp).reshape(16)
        _check(self.lib.dpcull_cull(self.h, g, r, fptr(v)))

    def result_changed(self, r: int, out: np.ndarray | None = None) -> np.ndarray:
        n = _SZ()
        if out is None:
            rc = self.lib.dpcull_result_changed(self.h, r, None, 0, C.byref(n))
            if rc not in (OK, ERR_CAPACITY):
                _check(rc)
            out = np.empty(max(n.value, 1), np.uint32)
        rc = self.lib.dpcull_result_changed(self.h, r, uptr(out), out.shape[0], C.byref(n))
        _check(rc)
        return out[: n.value]

    def result_read(self, r: int, bits: np.ndarray, changed: np.ndarray) -> int:
        """Visibility words into `bits` and the changed list into `changed` (uint32 arrays
        large enough) in one call; returns the changed-list length."""
        nb, nc = _SZ(), _SZ()
        _check(self.lib.dpcull_result_read(self.h, r, bits.ctypes.data, bits.size, C.byref(nb),
                                           changed.ctypes.data, changed.size, C.byref(nc)))
        return nc.value

    def result_bits(self, r: int, out: np.ndarray | None = None) -> np.ndarray:
        nb = _SZ()
        rc = self.lib.dpcull_result_bits(self.h, r, None, 0, C.byref(nb))
        if rc not in (OK, ERR_CAPACITY):
            _check(rc)
        words = (nb.value + 31) // 32
        if out is None:
            out = np.zeros(max(words, 1), np.uint32)
        _check(self.lib.dpcull_result_bits(self.h, r, uptr(out), out.shape[0], C.byref(nb)))
        return out[:words]

    def result_is_visible(self, r: int, index: int) -> bool:
        v = _I()
        _check(self.lib.dpcull_result_is_visible(self.h, r, index, C.byref(v)))
        return bool(v.value)

    def result_device(self, r: int):
        b, c, n = _P(), _P(), _P()
        _check(self.lib.dpcull_result_device(self.h, r, C.byref(b), C.byref(c), C.byref(n)))
        return b.value, c.value, n.value

    # ---- batched ----
    def _jobs(self, jobs):
        arr = (Job * len(jobs))()
        keep = []
        for i, (g, results, vps) in enumerate(jobs):
            rs = _u32(results)
            v = _f32(vps).reshape(-1, 16)
            assert v.shape[0] == rs.shape[0]
            keep += [rs, v]
            arr[i] = Job(g, rs.shape[0], uptr(rs), fptr(v))
        return arr, keep

    def cull_batched(self, jobs, tuning: dict | None = None) -> None:
        arr, keep = self._jobs(jobs)
        t = C.byref(Tuning(**tuning)) if tuning else None
        _check(self.lib.dpcull_cull_batched(self.h, arr, len(jobs), t))

    def autotune(self, jobs) -> dict:
        arr, keep = self._jobs(jobs)
        t = Tuning()
        _check(self.lib.dpcull_autotune(self.h, arr, len(jobs), C.byref(t)))
        return t.as_dict()

    def plan_create(self, jobs, tuning: dict | None = None) -> int:
        arr, keep = self._jobs(jobs)
        p = _U32()
        t = C.byref(Tuning(**tuning)) if tuning else None
        _check(self.lib.dpcull_plan_create(self.h, arr, len(jobs), t, C.byref(p)))
        return p.value

    def plan_set_views(self, p: int, vps) -> None:
        v = _f32(vps).reshape(-1)
        self._keep[("plan_vps", p)] = v
        _check(self.lib.dpcull_plan_set_views(self.h, p, fptr(v)))

    def plan_launch(self, p: int) -> None:
        _check(self.lib.dpcull_plan_launch(self.h, p))

    def plan_kernel_ms(self, p: int, back: int = 0) -> float:
        """Cull-kernel duration (ms) of the plan's last (back=0) or previous (back=1) launch."""
        ms = C.c_float()
        _check(self.lib.dpcull_plan_kernel_ms(self.h, p, back, C.byref(ms)))
        return ms.value

    def plan_read(self, p: int, bits: list, changed: list) -> np.ndarray:
        """Reads every result of the plan's last launch into the given uint32 arrays (one per
        result, in job and view order; None skips); returns the changed-list lengths."""
        n = len(bits)
        bp = (C.c_void_p * n)(*[(b.ctypes.data if b is not None else None) for b in bits])
        cp = (C.c_void_p * n)(*[(c.ctypes.data if c is not None else None) for c in changed])
        caps = (C.c_size_t * n)(*[(c.size if c is not None else 0) for c in changed])
        out = np.zeros(n, np.uint64)
        _check(self.lib.dpcull_plan_read(self.h, p, bp, cp, caps, out.ctypes.data))
        return out

    def plan_read_async(self, p: int, bits: list, changed: list) -> np.ndarray:
        """Starts reading every result of the plan's last launch into the given arrays (kept
        alive and untouched until plan_read_wait); returns the changed-list lengths."""
        n = len(bits)
        bp = (C.c_void_p * n)(*[(b.ctypes.data if b is not None else None) for b in bits])
        cp = (C.c_void_p * n)(*[(c.ctypes.data if c is not None else None) for c in changed])
        caps = (C.c_size_t * n)(*[(c.size if c is not None else 0) for c in changed])
        out = np.zeros(n, np.uint64)
        _check(self.lib.dpcull_plan_read_async(self.h, p, bp, cp, caps, out.ctypes.data))
        return out

    def plan_read_wait(self, p: int) -> None:
        _check(self.lib.dpcull_plan_read_wait(self.h, p))

    def plan_snapshot(self, p: int) -> None:
        """Snapshots the results of the plan's last launch without waiting; the next
        plan_read_async reads the snapshot (so the next launch can go out first)."""
        _check(self.lib.dpcull_plan_snapshot(self.h, p))

    def plan_tuning(self, p: int) -> dict:
        t = Tuning()
        _check(self.lib.dpcull_plan_tuning(self.h, p, C.byref(t)))
        return t.as_dict()

    def plan_destroy(self, p: int) -> None:
        _check(self.lib.dpcull_plan_destroy(self.h, p))

    # ---- transform tree ----
    def tree_create(self, capacity: int) -> int:
        t = _U32()
        _check(self.lib.dpcull_tree_create(self.h, capacity, C.byref(t)))
        return t.value

    def tree_destroy(self, t: int) -> None:
        _check(self.lib.dpcull_tree_destroy(self.h, t))

    def tree_resize(self, t: int, capacity: int) -> None:
        _check(self.lib.dpcull_tree_resize(self.h, t, capacity))

    def tree_set_structure(self, t: int, pairs, level_offsets) -> None:
        p = _u32(pairs).reshape(-1)
        lo = _u32(level_offsets)
        n_levels = max(lo.shape[0] - 1, 0)
        _check(self.lib.dpcull_tree_set_structure(self.h, t, p.shape[0] // 2, uptr(p), n_levels, uptr(lo)))

    def tree_set_locals(self, t: int, index, mats) -> None:
        ix, m = _u32(index), _f32(mats).reshape(-1, 16)
        _check(self.lib.dpcull_tree_set_locals(self.h, t, ix.shape[0], uptr(ix), fptr(m)))

    def tree_set_worlds(self, t: int, index, mats) -> None:
        ix, m = _u32(index), _f32(mats).reshape(-1, 16)
        _check(self.lib.dpcull_tree_set_worlds(self.h, t, ix.shape[0], uptr(ix), fptr(m)))

    def tree_compute(self, t: int) -> None:
        _check(self.lib.dpcull_tree_compute(self.h, t))

    def tree_world_device(self, t: int):
        p, n = _P(), _SZ()
        _check(self.lib.dpcull_tree_world_device(self.h, t, C.byref(p), C.byref(n)))
        return p.value, n.value

    def tree_world(self, t: int, first: int, count: int) -> np.ndarray:
        out = np.empty((count, 16), np.float32)
        _check(self.lib.dpcull_tree_world(self.h, t, first, count, fptr(out)))
        return out

    def tree_dirty_world(self, t: int, n_words: int) -> np.ndarray:
        out = np.zeros(n_words, np.uint32)
        _check(self.lib.dpcull_tree_dirty_world(self.h, t, uptr(out), n_words))
        return out


class Server:
    """A dpcull culling service (include/dpcull.h, serving section) on a context."""

    def __init__(self, ctx: Context, budget_bytes: int, n_streams: int = 3,
                 max_batch_objects: int = 32 << 20):
        self.ctx = ctx
        self.lib = ctx.lib
        h = _P()
        _check(self.lib.dpcull_server_create(ctx.h, int(budget_bytes), n_streams, int(max_batch_objects),
                                             C.byref(h)))
        self.h = h
        self._scenes: dict = {}  # host arrays stay alive while the server lives
        self._buf = (Completion * 4096)()

    def close(self) -> None:
        if self.h:
            _check(self.lib.dpcull_server_destroy(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def now(self) -> float:
        return float(self.lib.dpcull_server_now())

    def add_scene(self, scene: int, lower, extent, xform, mats) -> None:
        lo, ex, xf, m = _f32(lower), _f32(extent), _u32(xform), _f32(mats).reshape(-1, 16)
        self._scenes[scene] = (lo, ex, xf, m)
        _check(self.lib.dpcull_server_add_scene(self.h, scene, xf.shape[0], fptr(lo), fptr(ex), uptr(xf),
                                                fptr(m), m.shape[0]))

    def submit(self, scene: int, vps, keep_bits: bool = False) -> int:
        v = _f32(vps).reshape(-1)
        rid = C.c_uint64()
        _check(self.lib.dpcull_server_submit(self.h, scene, v.shape[0] // 16, fptr(v),
                                             REQUEST_KEEP_BITS if keep_bits else 0, C.byref(rid)))
        return rid.value

    def submit_raw(self, scene: int, n_views: int, vps_ptr, rid) -> int:
        """Low-overhead submit for load generators (pointer to n_views x 16 floats)."""
        return self.lib.dpcull_server_submit(self.h, scene, n_views, vps_ptr, 0, rid)

    def poll_array(self) -> np.ndarray:
        """All completions so far as a numpy structured array (fast path)."""
        parts = []
        while True:
            n = _SZ()
            _check(self.lib.dpcull_server_poll(self.h, self._buf, len(self._buf), C.byref(n)))
            if n.value:
                parts.append(np.ctypeslib.as_array(self._buf)[: n.value].copy())
            if n.value < len(self._buf):
                break
        if not parts:
            return np.ctypeslib.as_array(self._buf)[:0].copy()
        return np.concatenate(parts)

    def poll(self) -> list:
        a = self.poll_array()
        return [(int(c["request"]), int(c["scene"]), int(c["n_views"]), list(c["visible"][: c["n_views"]]),
                 int(c["objects"]), float(c["submit_s"]), float(c["start_s"]), float(c["done_s"]),
                 int(c["status"])) for c in a]

    def result(self, request: int, view: int, n_words: int) -> np.ndarray:
        out = np.zeros(n_words, np.uint32)
        _check(self.lib.dpcull_server_result(self.h, request, view, uptr(out), n_words))
        return out

    def release(self, request: int) -> None:
        _check(self.lib.dpcull_server_release(self.h, request))

    def drain(self) -> None:
        _check(self.lib.dpcull_server_drain(self.h))

    def stats(self) -> dict:
        st = ServerStats()
        _check(self.lib.dpcull_server_get_stats(self.h, C.byref(st)))
        return st.as_dict()
