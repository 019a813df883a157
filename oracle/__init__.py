"""Culling oracle -- TEST INFRASTRUCTURE ONLY.

ctypes access to two CPU implementations of the reference culling path with one handle
API (see cull_oracle.h):

* ``port()``      -- the C restatement in cull_oracle.c (``_build/liborc.so``), built
                     everywhere, including the GPU host;
* ``reference()`` -- the reference's own CPU manager and transform tree compiled from
                     the reference sources (``_ref/libdpref.so``), available only where
                     the reference tree exists.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference leg use
this package.  Nothing in pipeline_gb300/ imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liborc.so"
REF_LIB = HERE / "_ref" / "libdpref.so"
# The reference source tree: $DPCULL_REFERENCE, else a checkout named "reference" beside
# this repository.  Where neither exists the reference build and its tests are skipped.
REF_SRC = Path(os.environ.get("DPCULL_REFERENCE") or HERE.parent.parent / "reference")

_P, _I, _SZ, _U32, _U64, _I64 = C.c_void_p, C.c_int, C.c_size_t, C.c_uint32, C.c_uint64, C.c_int64
_FP, _UP, _IP = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_int)


def build(with_reference: bool | None = None) -> None:
    """make the port (always) and the reference harness (where its sources exist)."""
    targets = ["oracle"]
    if with_reference is None:
        with_reference = REF_SRC.is_dir()
    if with_reference:
        targets.append("ref")
    r = subprocess.run(["make", "-s", "-C", str(HERE), f"REF={REF_SRC}", *targets],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


def _sigs(p: str) -> dict:
    return {
        f"{p}mgr_create": (_P, []), f"{p}mgr_destroy": (None, [_P]),
        f"{p}object_create": (_I, [_P]),
        f"{p}object_set_bbox": (None, [_P, _I, _FP, _FP]),
        f"{p}object_set_xform": (None, [_P, _I, _U64]),
        f"{p}group_create": (_I, [_P]),
        f"{p}group_add": (_I, [_P, _I, _I]), f"{p}group_remove": (_I, [_P, _I, _I]),
        f"{p}group_count": (_SZ, [_P, _I]), f"{p}group_get_object": (_I, [_P, _I, _SZ]),
        f"{p}group_set_matrices": (None, [_P, _I, _P, _SZ, _SZ]),
        f"{p}group_matrix_changed": (None, [_P, _I, _SZ]),
        f"{p}result_create": (_I, [_P, _I]),
        f"{p}cull": (None, [_P, _I, _I, _FP]),
        f"{p}result_changed": (_SZ, [_P, _I, _IP, _SZ]),
        f"{p}result_is_visible": (_I, [_P, _I, _I]),
        f"{p}group_bbox": (None, [_P, _I, _FP, _FP]),
        f"{p}group_add_boxes": (_I, [_P, _I, _SZ, _FP, _FP, _UP]),
        f"{p}result_bits": (_SZ, [_P, _I, _UP, _SZ]),
        f"{p}tree_create": (_P, []), f"{p}tree_destroy": (None, [_P]),
        f"{p}tree_add": (_I64, [_P, _U32, _FP]), f"{p}tree_remove": (_I, [_P, _U32]),
        f"{p}tree_update_local": (None, [_P, _U32, _FP]),
        f"{p}tree_compute": (None, [_P]), f"{p}tree_count": (_SZ, [_P]),
        f"{p}tree_world": (_FP, [_P]),
        f"{p}tree_last_dirty": (_SZ, [_P, _UP, _SZ]),
    }


_PORT_ONLY = {
    "orc_vec4_mul_mat44": (None, [_FP, _FP, _FP]),
    "orc_mat44_mul": (None, [_FP, _FP, _FP]),
    "orc_build_obbs": (_I, [_SZ, _FP, _FP, _UP, _FP, _SZ, _FP]),
    "orc_cull_obbs": (None, [_SZ, _FP, _FP, _UP]),
    "orc_cull_obbs_mt": (None, [_I, _SZ, _FP, _FP, _UP]),
    "orc_cull_soa": (_I, [_SZ, _FP, _FP, _UP, _FP, _SZ, _FP, _UP]),
    "orc_update_changed": (_SZ, [_SZ, _UP, _UP, _UP]),
    "orc_bounding_box": (None, [_SZ, _FP, _FP, _UP, _FP, _FP, _FP]),
    "orc_propagate": (None, [_SZ, _UP, _FP, _FP, _UP, _UP]),
    "orc_tree_entries": (_SZ, [_P, _UP, _SZ, _UP, _SZ, C.POINTER(_SZ)]),
    "orc_tree_time_compute": (C.c_double, [_P, _UP, _SZ, _FP, _I, _I]),
}

_REF_ONLY = {
    "ref_time_cull": (C.c_double, [_P, _I, _I, _FP, _I, _I, _I, _SZ]),
    "ref_time_tree_compute": (C.c_double, [_P, _UP, _SZ, _FP, _I, _I]),
}


def _f(a):
    return np.ascontiguousarray(a, np.float32)


def _u(a):
    return np.ascontiguousarray(a, np.uint32)


def fp(a):
    return a.ctypes.data_as(_FP)


def up(a):
    return a.ctypes.data_as(_UP)


class CullLib:
    """Handle API common to the port and the reference build (prefix orc_ / ref_)."""

    def __init__(self, path: Path, prefix: str, extra: dict):
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (oracle.build())")
        self.lib = C.CDLL(str(path))
        self.prefix = prefix
        for name, (res, args) in {**_sigs(prefix), **extra}.items():
            f = getattr(self.lib, name)
            f.restype = res
            f.argtypes = args
        self._keep: list = []

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        return getattr(self.lib, self.prefix + name)

    # convenience wrappers ------------------------------------------------------------
    def manager(self):
        return Manager(self)

    def tree(self):
        return TreeHandle(self)


class Manager:
    """One dp::culling::Manager instance (port or reference)."""

    def __init__(self, lib: CullLib):
        self.L = lib
        self.h = lib.mgr_create()
        self._keep: dict = {}

    def __del__(self):
        try:
            self.L.mgr_destroy(self.h)
        except Exception:
            pass

    def group(self) -> int:
        return self.L.group_create(self.h)

    def result(self, g: int) -> int:
        return self.L.result_create(self.h, g)

    def add_boxes(self, g: int, lower, upper, xform) -> int:
        lo, hi, xf = _f(lower), _f(upper), _u(xform)
        return self.L.group_add_boxes(self.h, g, xf.shape[0], fp(lo), fp(hi), up(xf))

    def object_create(self) -> int:
        return self.L.object_create(self.h)

    def object_set_bbox(self, o: int, lower, upper) -> None:
        lo, hi = _f(lower), _f(upper)
        self.L.object_set_bbox(self.h, o, fp(lo), fp(hi))

    def object_set_xform(self, o: int, index: int) -> None:
        self.L.object_set_xform(self.h, o, index)

    def group_add(self, g: int, o: int) -> int:
        return self.L.group_add(self.h, g, o)

    def group_remove(self, g: int, o: int) -> int:
        return self.L.group_remove(self.h, g, o)

    def group_count(self, g: int) -> int:
        return self.L.group_count(self.h, g)

    def group_get_object(self, g: int, i: int) -> int:
        return self.L.group_get_object(self.h, g, i)

    def set_matrices(self, g: int, mats: np.ndarray, count: int | None = None, stride: int = 64) -> None:
        m = np.ascontiguousarray(mats)
        self._keep[g] = m  # the reference borrows the pointer
        n = m.shape[0] if count is None else count
        self.L.group_set_matrices(self.h, g, m.ctypes.data, n, stride)

    def matrix_changed(self, g: int, index: int) -> None:
        self.L.group_matrix_changed(self.h, g, index)

    def cull(self, g: int, r: int, vp) -> None:
        v = _f(vp).reshape(16)
        self.L.cull(self.h, g, r, fp(v))

    def changed(self, r: int) -> np.ndarray:
        n = self.L.result_changed(self.h, r, None, 0)
        out = np.zeros(max(n, 1), np.int32)
        self.L.result_changed(self.h, r, out.ctypes.data_as(_IP), n)
        return out[:n]

    def bits(self, r: int, n_words: int) -> np.ndarray:
        out = np.zeros(max(n_words, 1), np.uint32)
        self.L.result_bits(self.h, r, up(out), n_words)
        return out[:n_words]

    def is_visible(self, r: int, o: int) -> bool:
        return bool(self.L.result_is_visible(self.h, r, o))

    def bbox(self, g: int):
        lo, hi = np.zeros(3, np.float32), np.zeros(3, np.float32)
        self.L.group_bbox(self.h, g, fp(lo), fp(hi))
        return lo, hi


class TreeHandle:
    """One dp::transform::Tree instance (port or reference)."""

    def __init__(self, lib: CullLib):
        self.L = lib
        self.h = lib.tree_create()

    def __del__(self):
        try:
            self.L.tree_destroy(self.h)
        except Exception:
            pass

    def add(self, parent: int, m) -> int:
        return int(self.L.tree_add(self.h, parent, fp(_f(m).reshape(16))))

    def remove(self, index: int) -> int:
        return self.L.tree_remove(self.h, index)

    def update_local(self, index: int, m) -> None:
        self.L.tree_update_local(self.h, index, fp(_f(m).reshape(16)))

    def compute(self) -> None:
        self.L.tree_compute(self.h)

    def count(self) -> int:
        return int(self.L.tree_count(self.h))

    def world(self, n: int | None = None) -> np.ndarray:
        n = self.count() if n is None else n
        p = self.L.tree_world(self.h)
        return np.ctypeslib.as_array(p, shape=(n * 16,)).reshape(n, 16).copy()

    def last_dirty(self) -> np.ndarray:
        n = self.L.tree_last_dirty(self.h, None, 0)
        out = np.zeros(max(n, 1), np.uint32)
        self.L.tree_last_dirty(self.h, up(out), n)
        return out[:n]

    def entries(self):
        """Level lists (port only): (pairs [n,2], level_offsets [n_levels+1])."""
        nl = C.c_size_t()
        n = self.L.lib.orc_tree_entries(self.h, None, 0, None, 0, C.byref(nl))
        pairs = np.zeros(max(2 * n, 2), np.uint32)
        offs = np.zeros(nl.value + 1, np.uint32)
        self.L.lib.orc_tree_entries(self.h, up(pairs), n, up(offs), nl.value + 1, C.byref(nl))
        return pairs[: 2 * n].reshape(-1, 2), offs


_port = None
_ref = None


def port() -> CullLib:
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build(with_reference=False)
        _port = CullLib(PORT_LIB, "orc_", _PORT_ONLY)
    return _port


def reference() -> CullLib | None:
    """The reference build, or None where it cannot exist (no reference sources)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            if not REF_SRC.is_dir():
                return None
            build(with_reference=True)
        _ref = CullLib(REF_LIB, "ref_", _REF_ONLY)
    return _ref


# ---- stateless helpers on the port -------------------------------------------------------
def cull_bits(lower, extent, xform, mats, vp) -> np.ndarray:
    """Visibility words of one cull (OBB build + isVisible), port implementation."""
    L = port()
    lo, ex, xf, m, v = _f(lower), _f(extent), _u(xform), _f(mats).reshape(-1, 16), _f(vp).reshape(16)
    n = xf.shape[0]
    out = np.zeros(max((n + 31) // 32, 1), np.uint32)
    rc = L.lib.orc_cull_soa(n, fp(lo), fp(ex), up(xf), fp(m), m.shape[0], fp(v), up(out))
    if rc != 0:
        raise ValueError("transform index out of range")
    return out[: (n + 31) // 32]


def build_obbs(lower, extent, xform, mats) -> np.ndarray:
    L = port()
    lo, ex, xf, m = _f(lower), _f(extent), _u(xform), _f(mats).reshape(-1, 16)
    n = xf.shape[0]
    out = np.zeros((max(n, 1), 16), np.float32)
    if L.lib.orc_build_obbs(n, fp(lo), fp(ex), up(xf), fp(m), m.shape[0], fp(out)) != 0:
        raise ValueError("transform index out of range")
    return out[:n]


def cull_obbs(obbs, vp, threads: int = 1) -> np.ndarray:
    L = port()
    o, v = _f(obbs), _f(vp).reshape(16)
    n = o.shape[0]
    out = np.zeros(max((n + 31) // 32, 1), np.uint32)
    if threads > 1:
        L.lib.orc_cull_obbs_mt(threads, n, fp(o), fp(v), up(out))
    else:
        L.lib.orc_cull_obbs(n, fp(o), fp(v), up(out))
    return out[: (n + 31) // 32]


def update_changed(prev_bits: np.ndarray, vis_bits, n: int) -> np.ndarray:
    """ResultBitSet::updateChanged on arrays; prev_bits is updated in place."""
    L = port()
    vb = _u(vis_bits)
    out = np.zeros(max(n, 1), np.uint32)
    k = L.lib.orc_update_changed(n, up(prev_bits), up(vb), up(out))
    return out[:k]


def changed_list(prev_bits, new_bits, n: int) -> np.ndarray:
    """Ascending changed indices between two bit arrays (non-destructive)."""
    p = _u(prev_bits).copy()
    return update_changed(p, new_bits, n)


def bounding_box(lower, extent, xform, mats):
    L = port()
    lo, ex, xf, m = _f(lower), _f(extent), _u(xform), _f(mats).reshape(-1, 16)
    a, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
    L.lib.orc_bounding_box(xf.shape[0], fp(lo), fp(ex), up(xf), fp(m), fp(a), fp(b))
    return a, b


def time_tree_compute(pairs, locals_, warm: int = 2, reps: int = 10) -> float:
    """Median ms of the port's Tree::compute after updateLocalMatrix on every transform
    (the tree built by addTransform in the order of `pairs`, level by level)."""
    L = port()
    t = L.tree()
    for p, x in _u(pairs).reshape(-1, 2):
        got = t.add(int(p), locals_[x])
        if got != int(x):
            raise ValueError("pairs are not in addTransform order")
    ids = np.arange(1, locals_.shape[0], dtype=np.uint32)
    m = _f(locals_[1:])
    return float(L.lib.orc_tree_time_compute(t.h, up(ids), ids.shape[0], fp(m), warm, reps))


def propagate(pairs, local, world, dirty_local, dirty_world) -> None:
    """Tree::compute on arrays (world and dirty_world updated in place)."""
    L = port()
    p = _u(pairs).reshape(-1)
    L.lib.orc_propagate(p.shape[0] // 2, up(p), fp(local), fp(world), up(dirty_local), up(dirty_world))


def vec4_mul_mat44(v, m) -> np.ndarray:
    out = np.zeros(4, np.float32)
    port().lib.orc_vec4_mul_mat44(fp(_f(v)), fp(_f(m).reshape(16)), fp(out))
    return out


def mat44_mul(a, b) -> np.ndarray:
    out = np.zeros(16, np.float32)
    port().lib.orc_mat44_mul(fp(_f(a).reshape(16)), fp(_f(b).reshape(16)), fp(out))
    return out
