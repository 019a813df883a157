"""Serving workload: a catalogue of scenes and Poisson clients driving a dpcull server.

Catalogue: scene sizes log-uniform in [10k, 2M] objects, one shared world matrix per 16
objects (32 B per object resident), enough scenes that their resident bytes exceed the
HBM budget so that least-recently-used eviction runs.  To keep host memory and set-up
time bounded, the catalogue's scenes draw their data from a pool of generated templates
(scene k uses template k mod T); every catalogue scene is still a separate device
allocation, upload and eviction.

Clients: 64 independent Poisson streams totalling a mean arrival rate (default 20k
requests/s); each request culls one catalogue scene (uniformly chosen) under 1-6 views of
the client's camera rig (a perspective view, then cube faces), each jittered by up to 2
degrees.  Arrival times, scenes and view matrices are precomputed, so the submit loop only
waits for the arrival time and calls dpcull_server_submit.
"""
from __future__ import annotations

import ctypes as C
import gc
import math
import time

import numpy as np

from . import native
from . import workloads as W


def make_templates(seed: int, n_templates: int, nmin: float = 1e4, nmax: float = 2e6):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_templates):
        n = int(math.floor(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        n_m = max(1, n // 16)
        lower, upper, extent = W.random_boxes(rng, n)
        mats = W.random_matrices(rng, n_m)
        mats[:, 12:15] *= np.float32(0.3)  # scenes within +-300 of their origin
        xform = rng.integers(0, n_m, n, dtype=np.uint32)
        out.append(dict(lower=lower, extent=extent, xform=xform, mats=mats, n=n))
    return out


def scene_bytes(n: int, n_mats: int) -> int:
    cap = -(-n // 128) * 128
    return 7 * cap * 4 + 64 * n_mats


def random_rotations(rng: np.random.Generator, count: int, max_deg: float) -> np.ndarray:
    """count 4x4 rotations about random axes by angles uniform in [-max_deg, max_deg]."""
    axis = rng.standard_normal((count, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    ang = np.radians(rng.uniform(-max_deg, max_deg, count))
    K = np.zeros((count, 3, 3))
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 2] = -axis[:, 2], axis[:, 1], -axis[:, 0]
    K[:, 1, 0], K[:, 2, 0], K[:, 2, 1] = axis[:, 2], -axis[:, 1], axis[:, 0]
    I = np.eye(3)[None]
    R = I + np.sin(ang)[:, None, None] * K + (1 - np.cos(ang))[:, None, None] * (K @ K)
    out = np.zeros((count, 4, 4))
    out[:, :3, :3] = R
    out[:, 3, 3] = 1.0
    return out


def client_rigs(rng: np.random.Generator, n_clients: int) -> np.ndarray:
    """[client, 6, 4, 4]: a perspective view followed by 5 cube faces, per client."""
    rigs = np.zeros((n_clients, 6, 4, 4))
    for c in range(n_clients):
        eye = rng.uniform(-50, 50, 3)
        yaw = rng.uniform(0, 360)
        view = W.look_at(eye, eye + np.array([math.sin(math.radians(yaw)), 0.0, -math.cos(math.radians(yaw))]),
                         (0, 1, 0))
        rigs[c, 0] = view @ W.perspective()
        for k, v in enumerate(W.cube_face_views(eye)[:5]):
            rigs[c, k + 1] = v
    return rigs


def schedule(seed: int, n_scenes: int, duration_s: float, rate: float, n_clients: int = 64,
             max_views: int = 6):
    """Precomputed arrivals: times (s from start), scene ids, view counts, view matrices."""
    rng = np.random.default_rng(seed)
    rigs = client_rigs(rng, n_clients)
    per_client = rate / n_clients
    times, clients = [], []
    for c in range(n_clients):
        t = 0.0
        while True:
            t += rng.exponential(1.0 / per_client)
            if t >= duration_s:
                break
            times.append(t)
            clients.append(c)
    order = np.argsort(times)
    times = np.asarray(times)[order]
    clients = np.asarray(clients, np.int64)[order]
    m = len(times)
    scenes = rng.integers(0, n_scenes, m).astype(np.uint32)
    nviews = rng.integers(1, max_views + 1, m).astype(np.uint32)
    J = random_rotations(rng, m * max_views, 2.0).reshape(m, max_views, 4, 4)
    vps = np.einsum("mvij,mvjk->mvik", J, rigs[clients]).astype(np.float32).reshape(m, max_views, 16)
    return times, scenes, nviews, np.ascontiguousarray(vps)


def run_load(server: native.Server, times, scenes, nviews, vps, warmup_s: float = 0.0) -> dict:
    """Submits every request at its arrival time (relative to the start) and collects the
    completions.  Latency is measured from the scheduled arrival time."""
    lib = server.lib
    h = server.h
    rid = C.c_uint64()
    base = vps.ctypes.data
    stride = vps.strides[0]
    # A private handle to the same library whose submit takes the view pointer as a plain
    # address (no per-call pointer object).
    raw = C.CDLL(str(native.LIB_PATH))
    submit = raw.dpcull_server_submit
    submit.restype = C.c_int
    submit.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)]
    rid_ref = C.byref(rid)
    scenes_l = scenes.tolist()
    nviews_l = nviews.tolist()
    m = len(times)
    ids = np.zeros(m, np.uint64)
    done = []
    gc_was_on = gc.isenabled()
    gc.disable()  # no collector pauses inside the submission loop
    t0 = time.perf_counter()
    clock0 = server.now()
    late = 0
    for i in range(m):
        target = t0 + times[i]
        while True:
            now = time.perf_counter()
            if now >= target:
                break
            if target - now > 0.002:
                done.append(server.poll_array())
        if now - target > 0.001:
            late += 1
        rc = submit(h, scenes_l[i], nviews_l[i], base + i * stride, 0, rid_ref)
        if rc != 0:
            raise native.DpcullError(rc, lib.dpcull_last_error().decode())
        ids[i] = rid.value
    server.drain()
    wall = time.perf_counter() - t0
    if gc_was_on:
        gc.enable()
    done.append(server.poll_array())
    comp = np.concatenate(done)
    # request ids are consecutive in submission order
    index = (comp["request"] - ids[0]).astype(np.int64)
    arrival = clock0 + times[index]
    keep = arrival >= clock0 + warmup_s
    lat = (comp["done_s"][keep] - arrival[keep]) * 1e3
    ov = float(np.sum(comp["objects"][keep].astype(np.float64) * comp["n_views"][keep]))
    span = (clock0 + times[-1]) - (clock0 + warmup_s) if m else 1.0
    return {"requests": int(comp.shape[0]), "measured_requests": int(lat.size),
            "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
            "max_ms": float(lat.max()) if lat.size else None,
            "object_views_per_s": ov / max(span, 1e-9), "offered_rate": len(times) / max(times[-1], 1e-9),
            "late_submits": late, "wall_s": wall}
