"""Seeded synthetic culling workloads.

The reference ships no culling datasets (its render benchmarks load user-supplied
scene files), so the benchmark and test scenes are generated here with the shapes and
value distributions of the five benchmark configurations:

* ``plain_scene``   100k objects, one FP32 world matrix each (unit-quaternion rotation,
                    uniform scale in [0.5, 2], translation in [-1000, 1000]^3), local
                    boxes with centre in [-5, 5]^3 and extents in [0.1, 10]; perspective
                    60 deg, 16:9, near 0.1, far 5000, camera at the origin looking down
                    -Z, second frame yawed by 1 degree.
* ``hierarchy_scene`` 4M objects over 64k transforms of a tree of depth 8 with
                    branching 2-8, camera orbit of radius 800 (240 frames).
* ``batched_scenes`` 256 scenes of 1k-1M objects (log-uniform) with 1-6 views each
                    (perspective, orthographic shadow cascades, cube faces).
* ``stress_scene``  16M objects over 1M shared transforms, 8 views (6 cube faces and a
                    stereo pair with 6.5 cm eye separation).

Matrices follow the reference conventions (dp/math/Matmnt.h): 16 floats, row-major,
row-vector (clip = p * World * View * Projection).  Object boxes are returned both as
(lower, upper) -- what a caller hands to Manager::objectSetBoundingBox -- and as the
(lower, extent) pair the reference stores (extent = upper - lower in FP32,
dp/culling/src/ManagerBitSet.cpp:99-109).
"""
from __future__ import annotations

import math

import numpy as np

FOVY = 60.0
ASPECT = 16.0 / 9.0
NEAR = 0.1
FAR = 5000.0


# ---- matrix builders (row-vector convention) -----------------------------------------
def frustum(l, r, b, t, n, f) -> np.ndarray:
    """makeFrustum (dp/math/Matmnt.h:1315-1340) in row-vector form."""
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = 2 * n / (r - l)
    m[1, 1] = 2 * n / (t - b)
    m[2, 0] = (r + l) / (r - l)
    m[2, 1] = (t + b) / (t - b)
    m[2, 2] = -(f + n) / (f - n)
    m[2, 3] = -1.0
    m[3, 2] = -2 * f * n / (f - n)
    return m


def perspective(fovy=FOVY, aspect=ASPECT, near=NEAR, far=FAR) -> np.ndarray:
    """makePerspective (Matmnt.h:1354-1365)."""
    tanfov = math.tan(math.radians(fovy) * 0.5)
    r = tanfov * aspect * near
    t = tanfov * near
    return frustum(-r, r, -t, t, near, far)


def ortho(l, r, b, t, n, f) -> np.ndarray:
    """makeOrtho (Matmnt.h:1297-1308) in row-vector form."""
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = 2 / (r - l)
    m[1, 1] = 2 / (t - b)
    m[2, 2] = -2 / (f - n)
    m[3, 0] = -(r + l) / (r - l)
    m[3, 1] = -(t + b) / (t - b)
    m[3, 2] = -(f + n) / (f - n)
    m[3, 3] = 1.0
    return m


def look_at(eye, target, up) -> np.ndarray:
    """World-to-view matrix of a camera at `eye` looking at `target` (row-vector)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    fwd = target - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    back = -fwd
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2] = right, upv, back
    m[3, 0], m[3, 1], m[3, 2] = -right @ eye, -upv @ eye, -back @ eye
    return m


def rot_y(deg) -> np.ndarray:
    a = math.radians(deg)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = math.cos(a), -math.sin(a), math.sin(a), math.cos(a)
    return m


def f32(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float64).reshape(-1, 16).astype(np.float32))


# ---- objects and transforms ------------------------------------------------------------
def random_matrices(rng: np.random.Generator, n: int) -> np.ndarray:
    """setMat(q, t, (s,s,s)) (Matmnt.h:527-540): rows 0-2 = s * rotation rows (w = 0),
    row 3 = (t, 1); q a uniform unit quaternion (normalised 4-D Gaussian).  The rotation
    is evaluated in float64 and each entry rounded once to float32."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = (np.ascontiguousarray(q[:, i]) for i in range(4))
    s = rng.uniform(0.5, 2.0, n)
    t = rng.uniform(-1000.0, 1000.0, (n, 3))
    xx, yy, zz = x * x, y * y, z * z
    xy, xz, yz, zw, yw, xw = x * y, x * z, y * z, z * w, y * w, x * w
    rot = [1 - 2 * (yy + zz), 2 * (xy + zw), 2 * (xz - yw),
           2 * (xy - zw), 1 - 2 * (xx + zz), 2 * (yz + xw),
           2 * (xz + yw), 2 * (yz - xw), 1 - 2 * (xx + yy)]
    M = np.zeros((n, 16), np.float32)
    for k, r in enumerate(rot):
        i, j = divmod(k, 3)
        M[:, 4 * i + j] = r * s
    M[:, 12:15] = t
    M[:, 15] = 1.0
    return M


def random_boxes(rng: np.random.Generator, n: int):
    """Local boxes: centre in [-5,5]^3, extents in [0.1,10]^3, planar [3][n] float32.
    Returns (lower, upper, extent) with extent = upper - lower in FP32."""
    c = rng.uniform(-5.0, 5.0, (3, n))
    e = rng.uniform(0.1, 10.0, (3, n))
    lower = (c - 0.5 * e).astype(np.float32)
    upper = (c + 0.5 * e).astype(np.float32)
    extent = (upper - lower).astype(np.float32)
    return np.ascontiguousarray(lower), np.ascontiguousarray(upper), np.ascontiguousarray(extent)


def cube_face_views(eye=(0.0, 0.0, 0.0), near=NEAR, far=FAR) -> list[np.ndarray]:
    eye = np.asarray(eye, np.float64)
    P = perspective(90.0, 1.0, near, far)
    dirs = [((1, 0, 0), (0, -1, 0)), ((-1, 0, 0), (0, -1, 0)), ((0, 1, 0), (0, 0, 1)),
            ((0, -1, 0), (0, 0, -1)), ((0, 0, 1), (0, -1, 0)), ((0, 0, -1), (0, -1, 0))]
    return [look_at(eye, eye + np.asarray(d, np.float64), up) @ P for d, up in dirs]


def stereo_views(eye=(0.0, 0.0, 0.0), separation=0.065) -> list[np.ndarray]:
    P = perspective()
    out = []
    for s in (-0.5, 0.5):
        e = np.asarray(eye, np.float64) + np.array([s * separation, 0, 0])
        out.append(look_at(e, e + np.array([0, 0, -1.0]), (0, 1, 0)) @ P)
    return out


def cascade_views(n_cascades=4, light_dir=(-1.0, -2.0, -1.0), lam=0.5) -> list[np.ndarray]:
    """Orthographic shadow cascades covering splits of [NEAR, FAR] of the default camera
    (origin, looking down -Z), practical split scheme with weight `lam`."""
    d = np.asarray(light_dir, np.float64)
    d /= np.linalg.norm(d)
    splits = [NEAR]
    for i in range(1, n_cascades + 1):
        u = NEAR + (FAR - NEAR) * i / n_cascades
        lg = NEAR * (FAR / NEAR) ** (i / n_cascades)
        splits.append(lam * lg + (1 - lam) * u)
    tanv = math.tan(math.radians(FOVY) * 0.5)
    out = []
    for i in range(n_cascades):
        corners = []
        for z in (splits[i], splits[i + 1]):
            for sx in (-1, 1):
                for sy in (-1, 1):
                    corners.append((sx * tanv * ASPECT * z, sy * tanv * z, -z))
        corners = np.array(corners)
        centre = corners.mean(axis=0)
        radius = np.linalg.norm(corners - centre, axis=1).max()
        V = look_at(centre - d * (radius + 2000.0), centre, (0, 0, 1) if abs(d[1]) > 0.99 else (0, 1, 0))
        lc = np.c_[corners, np.ones(8)] @ V
        lo, hi = lc.min(axis=0), lc.max(axis=0)
        out.append(V @ ortho(lo[0], hi[0], lo[1], hi[1], -hi[2] - 10.0, -lo[2] + 2000.0))
    return out


# ---- configurations --------------------------------------------------------------------
def plain_scene(seed: int = 0, n: int = 100_000):
    """Two frames of one view over n objects, each with its own world matrix."""
    rng = np.random.default_rng(seed)
    lower, upper, extent = random_boxes(rng, n)
    mats = random_matrices(rng, n)
    P = perspective()
    vps = f32([np.eye(4) @ P, rot_y(-1.0) @ P])
    return dict(lower=lower, upper=upper, extent=extent, xform=np.arange(n, dtype=np.uint32),
                mats=mats, vps=vps)


def tree_levels(rng: np.random.Generator, n_transforms: int, depth: int = 8, bmin=2, bmax=8):
    """Breadth-first tree under the root (index 0): level lists of (parent, transform)
    pairs in creation order, as dp::transform::Tree builds them with addTransform
    (dp/transform/src/Tree.cpp:54-76; indices are allocated first-free, i.e. 1, 2, ...)."""
    pairs, offsets = [], [0]
    frontier = [0]
    nxt = 1
    for _ in range(depth):
        level = []
        for p in frontier:
            k = int(rng.integers(bmin, bmax + 1))
            for _ in range(k):
                if nxt >= n_transforms:
                    break
                level.append((p, nxt))
                nxt += 1
        if not level:
            break
        pairs += level
        offsets.append(len(pairs))
        frontier = [t for _, t in level]
        if nxt >= n_transforms:
            break
    return np.array(pairs, np.uint32).reshape(-1, 2), np.array(offsets, np.uint32), nxt


def hierarchy_scene(seed: int = 1, n_objects: int = 4_000_000, n_transforms: int = 65_536,
                    frames: int = 240, radius: float = 800.0):
    rng = np.random.default_rng(seed)
    pairs, offsets, used = tree_levels(rng, n_transforms)
    locals_ = random_matrices(rng, used)
    locals_[0] = np.eye(4, dtype=np.float32).reshape(16)
    lower, upper, extent = random_boxes(rng, n_objects)
    xform = rng.integers(0, used, n_objects, dtype=np.uint32)
    P = perspective()
    vps = []
    for f in range(frames):
        a = 2 * math.pi * f / frames
        eye = (radius * math.cos(a), 0.0, radius * math.sin(a))
        vps.append(look_at(eye, (0, 0, 0), (0, 1, 0)) @ P)
    return dict(pairs=pairs, level_offsets=offsets, n_transforms=used, locals=locals_,
                lower=lower, upper=upper, extent=extent, xform=xform, vps=f32(vps))


def scene_views(kind: str, n_views: int) -> list[np.ndarray]:
    if kind == "perspective":
        return [perspective()]
    if kind == "cascades":
        return cascade_views()[:n_views]
    return cube_face_views()[:n_views]


def batched_scenes(seed: int = 2, n_scenes: int = 256, nmin: float = 1e3, nmax: float = 1e6,
                   scale: float = 1.0, workers: int | None = None):
    """Scenes of uneven size (log-uniform object counts) with 1-6 views each:
    1 view = perspective, 2-4 = shadow cascades, 5-6 = cube faces.  Sizes and view counts
    come from one generator seeded with `seed`; each scene's boxes and matrices from its
    own child seed, so the scenes are generated in parallel (`workers` threads)."""
    import concurrent.futures as cf
    import os

    rng = np.random.default_rng(seed)
    sizes, counts = [], []
    for _ in range(n_scenes):
        n = int(math.floor(math.exp(rng.uniform(math.log(nmin), math.log(nmax))) * scale))
        sizes.append(max(n, 1))
        counts.append(int(rng.integers(1, 7)))
    children = np.random.SeedSequence(seed).spawn(n_scenes)

    def make(k: int) -> dict:
        r = np.random.default_rng(children[k])
        n, v = sizes[k], counts[k]
        kind = "perspective" if v == 1 else ("cascades" if v <= 4 else "cube")
        lower, upper, extent = random_boxes(r, n)
        mats = random_matrices(r, n)
        return dict(lower=lower, upper=upper, extent=extent, xform=np.arange(n, dtype=np.uint32),
                    mats=mats, vps=f32(scene_views(kind, v)), kind=kind)

    with cf.ThreadPoolExecutor(max_workers=workers or min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(make, range(n_scenes)))


STRESS_CHUNK = 1 << 20  # objects per independently seeded chunk of the stress scene


def stress_scene(seed: int = 3, n_objects: int = 16_000_000, n_transforms: int = 1_000_000,
                 begin: int = 0, end: int | None = None, workers: int | None = None):
    """The bandwidth stress scene, or the objects [begin, end) of it (a shard).  The
    shared world matrices come from `seed`; the objects are generated in chunks of
    STRESS_CHUNK objects, each from its own child seed, so a shard is generated without
    the rest of the scene (and the chunks in parallel): every rank of a multi-GPU run
    holds exactly its part of one global scene."""
    import concurrent.futures as cf
    import os

    end = n_objects if end is None else min(end, n_objects)
    rng = np.random.default_rng(seed)
    mats = random_matrices(rng, n_transforms)
    n_chunks = -(-n_objects // STRESS_CHUNK)
    seeds = np.random.SeedSequence([seed, 1]).spawn(n_chunks)
    n = max(end - begin, 0)
    lower = np.empty((3, n), np.float32)
    upper = np.empty((3, n), np.float32)
    extent = np.empty((3, n), np.float32)
    xform = np.empty(n, np.uint32)

    def fill(c: int) -> None:
        c0, c1 = c * STRESS_CHUNK, min(n_objects, (c + 1) * STRESS_CHUNK)
        lo, hi = max(c0, begin), min(c1, end)
        if lo >= hi:
            return
        r = np.random.default_rng(seeds[c])
        l_, u_, e_ = random_boxes(r, c1 - c0)
        x_ = r.integers(0, n_transforms, c1 - c0, dtype=np.uint32)
        a, b = lo - c0, hi - c0
        lower[:, lo - begin:hi - begin] = l_[:, a:b]
        upper[:, lo - begin:hi - begin] = u_[:, a:b]
        extent[:, lo - begin:hi - begin] = e_[:, a:b]
        xform[lo - begin:hi - begin] = x_[a:b]

    chunks = range(begin // STRESS_CHUNK, -(-end // STRESS_CHUNK)) if n else range(0)
    with cf.ThreadPoolExecutor(max_workers=workers or min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(fill, chunks))
    vps = f32(cube_face_views() + stereo_views())
    return dict(lower=lower, upper=upper, extent=extent, xform=xform, mats=mats, vps=vps, first=begin)


def jitter_view(rng: np.random.Generator, vp: np.ndarray, max_deg: float = 2.0) -> np.ndarray:
    """Rotates a view-projection by up to max_deg about a random axis (camera jitter)."""
    axis = rng.standard_normal(3)
    axis /= np.linalg.norm(axis)
    ang = math.radians(rng.uniform(-max_deg, max_deg))
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K
    J = np.eye(4)
    J[:3, :3] = R
    return f32(J @ np.asarray(vp, np.float64).reshape(4, 4))[0]
