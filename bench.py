"""Culling benchmark: culled object-views/s of the batched persistent CUDA path (bit-exact),
next to the plain per-call path, the roofline of the cull kernel, end-to-end throughput
through the C ABI with host buffers, and the reference CPU path on the host cores.

Default workload (the bandwidth stress configuration): 16M objects over 1M shared world
matrices, 8 simultaneous views (6 cube faces + a stereo pair), seeded synthetic data.  A
step is one batched cull of all objects in all views under a new camera (jittered by up
to 2 degrees per step, so the changed lists are not empty).  Objects and matrices do not
change between steps, so from the second launch on the kernel reads each group's box cache
(the counterpart of the reference's OBB cache, which its CPU manager likewise keeps until
an object or a matrix changes); the "cold" leg times the same steps with the cache off
(every launch transforms every object's box, the work of a frame whose matrices all changed).
The default line also carries the plain, hierarchy and batched configurations ("configs").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload stress|plain|hierarchy|batched|serving] [--no-configs]

N > 1 runs under torch.distributed.run, one process per GPU: the global scene has
N x 16M objects and every rank culls its contiguous shard (weak scaling, no data-path
collective); the barrier and the max over ranks of the timed region use torch.distributed,
and the end-to-end leg gathers every rank's words and changed lists to rank 0 (gloo) and
merges them into the whole scene's.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from pipeline_gb300 import workloads as W  # noqa: E402

STRESS_N, STRESS_T = 16_000_000, 1_000_000
METRIC = "culled object-views/s (batched persistent launch, bit-exact vs reference CPU manager)"


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ---- distributed plumbing ----------------------------------------------------------------
class Dist:
    def __init__(self, want: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.host = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            torch.cuda.set_device(self.local)
            dist.init_process_group("nccl")
            self.pg = dist
            self.host = dist.new_group(backend="gloo")  # result assembly on host tensors

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{self.local}")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks --------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        exe = shutil.which("nvidia-smi")
        if not exe:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen([exe, f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits", "-lms", "200"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        time.sleep(0.3)

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---- workloads -------------------------------------------------------------------------------
def make_frames(rng, base_vps, steps):
    """One view set per step: the base views, each rotated by up to 2 degrees."""
    return [np.stack([W.jitter_view(rng, v) for v in base_vps]) for _ in range(steps)]


class Stress:
    """The stress scene, or rank `rank`'s shard of a global scene of `world` x n objects
    (contiguous, 32-aligned object ranges; every rank holds the shared matrices)."""
    name = "stress"

    def __init__(self, seed: int, n: int = STRESS_N, t: int = STRESS_T, world: int = 1, rank: int = 0,
                 end: int | None = None):
        from pipeline_gb300 import shard

        self.n_total = n * world
        b, e = shard.shard_bounds(self.n_total, world, rank)
        if end is not None:  # a prefix of the scene (the CPU baseline's sample)
            b, e = 0, min(end, self.n_total)
        self.sc = W.stress_scene(seed=seed, n_objects=self.n_total, n_transforms=t, begin=b, end=e)
        self.first = b
        self.n, self.t, self.v = e - b, t, self.sc["vps"].shape[0]
        self.describe = (f"bandwidth stress: {n // 1_000_000}M objects per GPU over {t // 1_000_000}M shared "
                         f"world matrices (index uniform), {self.v} views (6 cube faces + stereo pair, 6.5 cm), "
                         "FP32 SoA, new camera per step (jitter <= 2 deg)")

    def setup(self, ctx, tuning=None):
        from pipeline_gb300 import native  # noqa: F401

        sc = self.sc
        self.g = ctx.group_create()
        ctx.group_set_objects(self.g, sc["lower"], sc["extent"], sc["xform"])
        ctx.group_set_matrices(self.g, sc["mats"])
        self.rs = [ctx.result_create(self.g) for _ in range(self.v)]
        self.rp = [ctx.result_create(self.g) for _ in range(self.v)]
        self.plan = ctx.plan_create([(self.g, self.rs, sc["vps"])], tuning)
        self.referenced = int(np.unique(sc["xform"]).size)

    def object_views(self) -> int:
        return self.n * self.v

    def algorithmic_bytes(self, changed_total: int) -> int:
        words = (self.n + 31) // 32
        return (28 * self.n + 64 * self.referenced + 64 * self.v + self.v * words * 4 * 2
                + 4 * changed_total)


def parse_tuning(s: str | None) -> dict | None:
    """JSON, or 'views_per_pass,tiles_per_ticket,ctas_per_sm'; None = run the autotuner."""
    if not s:
        return None
    if s.strip().startswith("{"):
        return json.loads(s)
    a, b, c = (int(x) for x in s.split(","))
    return {"views_per_pass": a, "tiles_per_ticket": b, "ctas_per_sm": c}


# ---- our arm ---------------------------------------------------------------------------------
def run_ours(args, dist: Dist) -> dict | None:
    import torch

    from pipeline_gb300 import build, native

    if dist.rank == 0 or not (ROOT / "pipeline_gb300" / "_lib" / "libdpcull.so").exists():
        build.build_all()
    dist.barrier()
    device = dist.local
    torch.cuda.set_device(device)
    wl = Stress(seed=3, n=args.objects, t=args.transforms, world=dist.world, rank=dist.rank)
    ctx = native.Context(device)
    if args.exact_only:
        ctx.set_prefilter(False)
    if args.no_box_cache:
        ctx.set_box_cache(False)
    wl.setup(ctx, parse_tuning(args.tuning))
    tuning = ctx.plan_tuning(wl.plan)
    rng = np.random.default_rng(17)  # one camera path for the whole (global) scene
    frames = make_frames(rng, wl.sc["vps"], args.warmup + args.steps + 1)
    stream = torch.cuda.ExternalStream(ctx.stream)

    # -- batched persistent path (graph replay), device-resident inputs --
    for i in range(args.warmup):
        ctx.plan_set_views(wl.plan, frames[i])
        ctx.plan_launch(wl.plan)
    ctx.synchronize()
    # Two events bracket the timed steps: an event recorded between graph launches costs
    # ~2 us of device time per step, so the per-step latencies come from a separate loop.
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    clocks = Clocks(device)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.kernel_launches
    kinds0 = ctx.cull_launches()
    kernel_ms = []
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(args.steps):
            ctx.plan_set_views(wl.plan, frames[args.warmup + i])
            ctx.plan_launch(wl.plan)
            if i:  # the cull kernel of the previous step (events inside the plan's graph)
                kernel_ms.append(ctx.plan_kernel_ms(wl.plan, 1))
        ev[1].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    kernel_ms.append(ctx.plan_kernel_ms(wl.plan, 0))
    launches = ctx.kernel_launches - launches0
    kinds = {k: v - kinds0[k] for k, v in ctx.cull_launches().items()}
    clk = clocks.stop()
    total_ms = ev[0].elapsed_time(ev[1])
    total_ms = dist.max(total_ms)
    # per-step latencies: the last timed steps again, an event after each (ending on the
    # last timed step's camera, which the parity sample below checks)
    lat_steps = min(args.steps, 100)
    lev = [torch.cuda.Event(enable_timing=True) for _ in range(lat_steps + 1)]
    with torch.cuda.stream(stream):
        lev[0].record(stream)
        for i in range(lat_steps):
            ctx.plan_set_views(wl.plan, frames[args.warmup + args.steps - lat_steps + i])
            ctx.plan_launch(wl.plan)
            lev[i + 1].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    step_ms = [lev[i].elapsed_time(lev[i + 1]) for i in range(lat_steps)]
    dist.barrier()
    changed = [len(ctx.result_changed(r)) for r in wl.rs]
    ms_step = total_ms / args.steps
    value = wl.object_views() * dist.world / (ms_step / 1e3)

    # -- plain per-call path: one launch per view and cull call --
    for i in range(2):
        for v in range(wl.v):
            ctx.cull(wl.g, wl.rp[v], frames[i][v])
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_steps = max(3, min(args.steps, 20))
    with torch.cuda.stream(stream):
        e0.record(stream)
        for i in range(plain_steps):
            for v in range(wl.v):
                ctx.cull(wl.g, wl.rp[v], frames[args.warmup + i][v])
        e1.record(stream)
    ctx.synchronize()
    plain_ms = dist.max(e0.elapsed_time(e1) / plain_steps)

    # -- parity spot check after the timed region: every view, first 256k objects --
    parity = parity_sample(ctx, wl, frames[args.warmup + args.steps - 1])

    # -- cold: the same steps with the box cache off (every box transformed every launch) --
    cold = None if args.no_box_cache else run_cold(ctx, wl, frames, args, dist, stream)

    # -- end to end through the C ABI with host buffers --
    e2e = run_e2e(ctx, wl, frames, args, dist)

    # -- serving loop (device-resident catalogue, continuous batching) --
    serving_res = None
    if args.serve_seconds > 0 and dist.rank == 0:
        # free the stress scene, its plan and results before filling the budget
        ctx.plan_destroy(wl.plan)
        for r in wl.rs + wl.rp:
            ctx.result_destroy(r)
        ctx.group_destroy(wl.g)
        torch.cuda.empty_cache()
        import gc

        gc.collect()  # no collection of the earlier legs' arrays inside the latency window
        serving_res = run_serving(ctx, args)

    # -- the other configurations, one GPU each (rank 0) --
    configs = None
    if not args.no_configs and dist.rank == 0:
        configs = {"cfg0_plain": run_plain_config(ctx, args), "cfg1_hierarchy": run_hierarchy_config(ctx, args),
                   "cfg2_batched": run_batched_config(ctx, args)}

    bytes_launch = wl.algorithmic_bytes(sum(changed))
    pk = peaks()
    k_ms = float(np.mean(kernel_ms))
    achieved = bytes_launch / (k_ms / 1e3) / 1e9
    traffic = traffic_from_profile(wl)
    bounds = issue_roofline(wl, k_ms, (clk or {}).get("sm_mhz"))
    if cold is not None:
        cb = issue_roofline(wl, cold["roofline"]["kernel_ms"], (clk or {}).get("sm_mhz"), "cold")
        cold["roofline"]["issue"], cold["roofline"]["fp32"] = cb
    out = {
        "metric": METRIC,
        "value": value, "unit": "object-views/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; the reference publishes no dataset)",
        "config": {"workload": wl.describe, "objects_per_gpu": wl.n, "objects_total": wl.n_total,
                   "transforms": wl.t, "views": wl.v,
                   "parallelism": f"{dist.world} contiguous object shards of one scene (no data-path collective)",
                   "l2": "no flush: per-step object data (448 MB; 320 MB of box cache when warm) exceeds L2 (126 MB)",
                   "box_cache": ("off" if args.no_box_cache else
                                 "on: launch 1 transforms the boxes and stores them, later launches read them "
                                 "(objects and matrices unchanged); the cold leg has it off"),
                   "tuning": tuning},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                       "max": float(max(step_ms)), "steps": lat_steps,
                       "note": "a separate loop over the last timed steps with an event after each"},
        "plain": {"value": wl.object_views() * dist.world / (plain_ms / 1e3), "ms_per_step": plain_ms,
                  "launches_per_step": wl.v},
        "batched_vs_plain": plain_ms / ms_step,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "peak_source": pk["source"], "algorithmic_bytes_per_launch": bytes_launch,
                     "kernel_ms": k_ms, "step_ms": ms_step,
                     "kernel": "cull_kernel: CUDA events recorded inside the plan graph right before "
                               "and after the kernel, every timed step",
                     "issue": bounds[0], "fp32": bounds[1]},
        "cold": cold, "e2e": e2e, "gpu_launches": launches, "cull_kernels_timed": kinds, "clocks": clk, "parity_sample": parity,
        "changed_per_step": changed, "configs": configs, "serving": serving_res,
    }
    ctx.close()
    return out


def parity_sample(ctx, wl, vps, m: int = 262_144) -> dict:
    import oracle

    sc = wl.sc
    obbs = oracle.build_obbs(sc["lower"][:, :m], sc["extent"][:, :m], sc["xform"][:m], sc["mats"])
    ok = True
    for v, r in enumerate(wl.rs):
        gpu = ctx.result_bits(r)[: m // 32]
        ok &= bool(np.array_equal(gpu, oracle.cull_obbs(obbs, vps[v], threads=8)))
    return {"objects": m, "views": len(wl.rs), "bit_exact": ok}


def run_cold(ctx, wl, frames, args, dist, stream) -> dict:
    """The timed steps again with the box cache off: every launch reads every object's box
    and transform index and gathers its world matrix (the fused kernel), as in a frame
    in which every matrix changed."""
    import torch

    ctx.set_box_cache(False)
    kinds0 = ctx.cull_launches()
    for i in range(args.warmup):
        ctx.plan_set_views(wl.plan, frames[i])
        ctx.plan_launch(wl.plan)
    ctx.synchronize()
    steps = max(3, min(args.steps, 50))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    kernel_ms = []
    dist.barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(steps):
            ctx.plan_set_views(wl.plan, frames[args.warmup + i])
            ctx.plan_launch(wl.plan)
            if i:
                kernel_ms.append(ctx.plan_kernel_ms(wl.plan, 1))
        ev[1].record(stream)
    ctx.synchronize()
    kernel_ms.append(ctx.plan_kernel_ms(wl.plan, 0))
    ms_step = dist.max(ev[0].elapsed_time(ev[1]) / steps)
    kinds = {k: v - kinds0[k] for k, v in ctx.cull_launches().items()}
    ctx.set_box_cache(True)
    changed = [len(ctx.result_changed(r)) for r in wl.rs]
    k_ms = float(np.mean(kernel_ms))
    bytes_launch = wl.algorithmic_bytes(sum(changed))
    pk = peaks()
    achieved = bytes_launch / (k_ms / 1e3) / 1e9
    return {"value": wl.object_views() * dist.world / (ms_step / 1e3), "unit": "object-views/s",
            "ms_per_step": ms_step, "steps": steps, "cull_kernels": kinds,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / pk["hbm_gbs"], "peak_source": pk["source"],
                         "traffic": _profile_scaled(wl, "dram_bytes_per_launch", "cold"),
                         "algorithmic_bytes_per_launch": bytes_launch, "kernel_ms": k_ms,
                         "kernel": "cull_kernel, fused (no box cache): CUDA events inside the plan graph"}}


def run_e2e(ctx, wl, frames, args, dist) -> dict:
    """Steps through the public API with host buffers: H2D of the step's view matrices from
    pinned memory, the batched cull, D2H of every view's visibility words and changed list.
    With N > 1 ranks every step's results are also gathered to rank 0 and merged into the
    whole scene's words and changed lists (host tensors over gloo)."""
    import torch

    from pipeline_gb300 import shard

    words = (wl.n + 31) // 32
    bits = [torch.empty(words, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
            for _ in range(wl.v)]
    changed = [torch.empty(max(wl.n, 1), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
               for _ in range(wl.v)]
    vps_pinned = torch.empty((wl.v, 16), dtype=torch.float32, pin_memory=True).numpy()
    # at least 100 steps: the pipeline's start (no copies to overlap yet) and its end (the
    # last step's copies, waited for) fall inside the timed region
    steps = max(100, min(args.steps, 400))
    d2h = 0
    merged = None

    def assemble(n_ch):
        if dist.world > 1:
            return shard.gather_results(bits, changed, n_ch, wl.n, wl.first, group=dist.host)
        return None

    dist.barrier()
    t0 = time.perf_counter()
    for i in range(steps):
        vps_pinned[:] = frames[i % len(frames)]
        ctx.plan_set_views(wl.plan, vps_pinned)
        if i:
            ctx.plan_snapshot(wl.plan)  # step i-1's results, before step i overwrites them
        ctx.plan_launch(wl.plan)
        if i:
            ctx.plan_read_wait(wl.plan)  # step i-2's results are on the host
            if i > 1:
                merged = assemble(n_ch)
            # step i-1's results: copies overlap step i's cull, which is already queued
            n_ch = ctx.plan_read_async(wl.plan, bits, changed)
            d2h += wl.v * (words * 4 + 4) + 4 * int(n_ch.sum())
    ctx.plan_read_wait(wl.plan)
    if steps > 1:
        merged = assemble(n_ch)
    n_ch = ctx.plan_read_async(wl.plan, bits, changed)  # the last step's results
    d2h += wl.v * (words * 4 + 4) + 4 * int(n_ch.sum())
    ctx.plan_read_wait(wl.plan)
    merged = assemble(n_ch)
    dt = dist.max(time.perf_counter() - t0)
    out = {"value": wl.object_views() * dist.world * steps / dt, "unit": "object-views/s",
           "ms_per_step": dt * 1e3 / steps, "h2d_bytes_per_step": wl.v * 64,
           "d2h_bytes_per_step": int(d2h / steps), "steps": steps,
           "path": "plan_set_views + plan_snapshot + plan_launch + plan_read_async / plan_read_wait "
                   "(every view's words and changed list of the previous step, copied while this "
                   "step culls; C ABI)"}
    if dist.world > 1:
        out["assembly"] = "every step: all ranks' words and changed lists gathered to rank 0 over gloo and merged"
        if merged is not None:
            out["merged_words_per_view"] = int(merged[0][0].size)
    return out


def _profile_scaled(wl, key: str, kernel: str = "warm") -> int | None:
    """A per-launch count from the committed ncu summary of the stress kernel (the warm
    kernel reading the box cache, or the cold fused one), scaled to this workload by
    object-views."""
    p = ROOT / "profiles" / "cull_stress_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(kernel)
    if not d or key not in d:
        return None
    scale = (wl.n * wl.v) / (d["objects"] * d["views"])
    return int(d[key] * scale)


def traffic_from_profile(wl, kernel: str = "warm") -> int | None:
    """DRAM bytes per launch from the committed ncu summary, scaled to this workload."""
    return _profile_scaled(wl, "dram_bytes_per_launch", kernel)


def issue_roofline(wl, k_ms: float, sm_mhz, kernel: str = "warm") -> tuple[dict | None, dict | None]:
    """The cull kernel's compute bounds (pipe_bounds) on this GPU."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return pipe_bounds(wl, k_ms, sm_mhz, sms, kernel)


def pipe_bounds(wl, k_ms: float, sm_mhz, sms: int, kernel: str = "warm") -> tuple[dict | None, dict | None]:
    """The cull kernel's two compute bounds beside HBM: warp-instruction issue (one per
    scheduler, 4 per SM, per cycle) and FP32 lane operations (128 lanes per SM per cycle).
    The counts per launch come from the committed ncu capture (scaled by object-views), the
    duration from this run's in-graph events, the clock is the median sampled during the
    timed region."""
    inst = _profile_scaled(wl, "warp_instructions_per_launch", kernel)
    if inst is None or not sm_mhz or not k_ms:
        return None, None
    secs = k_ms / 1e3
    achieved = inst / secs / 1e9
    peak = sms * 4 * float(sm_mhz) * 1e6 / 1e9
    issue = {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "G warp-instructions/s",
             "frac": achieved / peak, "warp_instructions_per_launch": inst,
             "thread_instructions_per_object_view": inst * 32 / wl.object_views(),
             "note": "instruction count from profiles/cull_stress_traffic.json scaled by object-views; "
                     "peak = SMs x 4 schedulers x median sampled SM clock"}
    ops = _profile_scaled(wl, "fp32_lane_ops_per_launch", kernel)
    fp32 = None
    if ops is not None:
        a = ops / secs / 1e12
        p = sms * 128 * float(sm_mhz) * 1e6 / 1e12
        fp32 = {"bound": "fp32", "achieved": a, "peak": p, "unit": "T FP32 lane-ops/s", "frac": a / p,
                "ops_per_object_view": ops / wl.object_views(),
                "note": "FFMA, FADD and FMUL count one lane-op, FFMA2 two (ncu opcode counts in "
                        "profiles/cull_stress_traffic.json); peak = SMs x 128 FP32 lanes x median sampled "
                        "SM clock"}
    return issue, fp32


# ---- other configurations (separate JSON lines; not the headline) ------------------------------
def _events(torch, n):
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def run_plain_config(ctx, args) -> dict:
    """Plain configuration: 100k objects with their own matrices, one view; a step is one
    dpcull_cull plus the changed list and the visibility words read back (the reference's
    cull call), alternating two frames 1 degree apart."""
    import torch

    sc = W.plain_scene(0, 100_000)
    g = ctx.group_create()
    ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
    ctx.group_set_matrices(g, sc["mats"])
    r = ctx.result_create(g)
    bits = np.zeros(3125, np.uint32)
    changed = np.zeros(100_000, np.uint32)
    for i in range(args.warmup):
        ctx.cull(g, r, sc["vps"][i % 2])
        ctx.result_changed(r, changed)
    lat = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        ctx.cull(g, r, sc["vps"][i % 2])
        ctx.result_read(r, bits, changed)  # changed list and visibility words, one call
        lat.append(time.perf_counter() - t0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    ev = _events(torch, 2)
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(args.steps):
            ctx.cull(g, r, sc["vps"][i % 2])
        ev[1].record(stream)
    ctx.synchronize()
    dev_ms = ev[0].elapsed_time(ev[1]) / args.steps
    lat = np.asarray(lat) * 1e3
    import oracle

    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    prev = np.zeros(3125, np.uint32)
    ts = []
    for i in range(9):
        t0 = time.perf_counter()
        b = oracle.cull_obbs(obbs, sc["vps"][i % 2])
        oracle.update_changed(prev, b, 100_000)
        ts.append(time.perf_counter() - t0)
    cpu_ms = sorted(ts)[4] * 1e3
    ctx.group_destroy(g)
    return {"workload": "plain: 100k objects, own matrices, 1 view, 2 frames 1 deg apart",
            "device_ms_per_cull": dev_ms, "object_views_per_s_device": 100_000 / (dev_ms / 1e3),
            "e2e_p50_ms": float(np.percentile(lat, 50)), "e2e_p99_ms": float(np.percentile(lat, 99)),
            "object_views_per_s_e2e": 100_000 / (np.median(lat) / 1e3),
            "cpu_port_1core_ms": cpu_ms, "cpu_object_views_per_s": 100_000 / (cpu_ms / 1e3)}


def run_hierarchy_config(ctx, args) -> dict:
    """Hierarchy configuration: 4M objects over 64k transforms of a depth-8 tree; every
    frame uploads all local matrices (animated), propagates them on the GPU and culls
    through the device world matrices under the next camera of a radius-800 orbit."""
    import torch

    from pipeline_gb300.transform import Tree

    sc = W.hierarchy_scene(seed=1, frames=240)
    used = sc["n_transforms"]
    t = Tree(ctx)
    for p, x in sc["pairs"]:
        t.add_transform(int(p), sc["locals"][x])
    t.compute()
    dev, count = t.world_device()
    g = ctx.group_create()
    ctx.group_set_objects(g, sc["lower"], sc["extent"], sc["xform"])
    ctx.group_bind_device_matrices(g, dev, count)
    r = ctx.result_create(g)
    # the per-frame inputs live in page-locked host memory, as an animation system's
    # output buffers would: each upload is then one DMA (no host staging copy)
    import torch

    idx = torch.empty(used - 1, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    idx[:] = np.arange(1, used, dtype=np.uint32)
    locs = torch.empty(sc["locals"][1:].shape, dtype=torch.float32, pin_memory=True).numpy()
    locs[:] = sc["locals"][1:]
    stream = torch.cuda.ExternalStream(ctx.stream)
    frames = sc["vps"].shape[0]
    for i in range(args.warmup):
        ctx.tree_set_locals(t.handle, idx, locs)
        ctx.tree_compute(t.handle)
        ctx.cull(g, r, sc["vps"][i % frames])
    ctx.synchronize()
    ev = _events(torch, 4)
    n = min(args.steps, frames)
    up_ms = prop_ms = cull_ms = 0.0
    t0 = time.perf_counter()
    for i in range(n):
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            u0 = time.perf_counter()
            ctx.tree_set_locals(t.handle, idx, locs)  # H2D from page-locked memory + scatter (dirty bits)
            up_ms += (time.perf_counter() - u0) * 1e3
            ev[1].record(stream)
            ctx.tree_compute(t.handle)
            ev[2].record(stream)
            ctx.cull(g, r, sc["vps"][i % frames])
            ev[3].record(stream)
        ch = ctx.result_changed(r)
        prop_ms += ev[1].elapsed_time(ev[2])
        cull_ms += ev[2].elapsed_time(ev[3])
    wall_ms = (time.perf_counter() - t0) * 1e3 / n
    ctx.group_destroy(g)
    ctx.tree_destroy(t.handle)
    import oracle

    # the reference's Tree::compute (all transforms dirty), single thread on the host
    cpu_ms = oracle.time_tree_compute(sc["pairs"], sc["locals"])
    p_ms = prop_ms / n
    pk = peaks()
    prop_bytes = 132 * (used - 1)  # local read 64 + parent index 4 + world write 64 per transform
    achieved = prop_bytes / (p_ms / 1e3) / 1e9
    return {"workload": f"hierarchy: 4M objects, {used} transforms (depth 8, branching 2-8), orbit r=800",
            "frames": n, "ms_per_frame_e2e": wall_ms, "upload_locals_host_ms": up_ms / n,
            "propagate_ms": p_ms, "cull_ms": cull_ms / n,
            "propagate_transforms_per_s": (used - 1) / (p_ms / 1e3),
            "cpu_tree_compute_ms": cpu_ms, "propagate_vs_cpu": cpu_ms / p_ms,
            "propagate_roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                                   "frac": achieved / pk["hbm_gbs"], "peak_source": pk["source"],
                                   "algorithmic_bytes": prop_bytes,
                                   "note": "132 B per transform over one propagation (one cooperative launch); "
                                           "an 8.6 MB working set is latency-bound, not HBM-bound"},
            "object_views_per_s_e2e": 4_000_000 / (wall_ms / 1e3),
            "note": "per frame: all 64k local matrices updated from page-locked host memory (4 MB), GPU propagation, "
                    "cull through the device world matrices, changed list read back; cpu_tree_compute_ms = "
                    "the oracle's Tree::compute restatement over the same tree, all transforms dirty, 1 thread"}


def run_batched_config(ctx, args) -> dict:
    """Batched-uneven configuration: 256 scenes of 1k-1M objects (log-uniform) with 1-6
    views each; one captured persistent plan vs one plain launch per scene and view."""
    import torch

    scenes = W.batched_scenes(seed=2)
    jobs, plain = [], []
    ov = 0
    for s in scenes:
        g = ctx.group_create()
        ctx.group_set_objects(g, s["lower"], s["extent"], s["xform"])
        ctx.group_set_matrices(g, s["mats"])
        jobs.append((g, [ctx.result_create(g) for _ in s["vps"]], s["vps"]))
        plain.append((g, [ctx.result_create(g) for _ in s["vps"]], s["vps"]))
        ov += len(s["xform"]) * len(s["vps"])
    p = ctx.plan_create(jobs)
    tuning = ctx.plan_tuning(p)
    stream = torch.cuda.ExternalStream(ctx.stream)
    for _ in range(args.warmup):
        ctx.plan_launch(p)
    ctx.synchronize()
    ev = _events(torch, 4)
    n = max(3, min(args.steps, 50))
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for _ in range(n):
            ctx.plan_launch(p)
        ev[1].record(stream)
    ctx.synchronize()
    batched_ms = ev[0].elapsed_time(ev[1]) / n
    with torch.cuda.stream(stream):
        ev[2].record(stream)
        for _ in range(n):
            for g, rs, vps in plain:
                for rr, vp in zip(rs, vps):
                    ctx.cull(g, rr, vp)
        ev[3].record(stream)
    ctx.synchronize()
    plain_ms = ev[2].elapsed_time(ev[3]) / n
    ctx.plan_destroy(p)
    for g, _, _ in jobs:
        ctx.group_destroy(g)
    return {"workload": f"batched uneven: 256 scenes, {sum(len(s['xform']) for s in scenes)} objects, "
                        f"{sum(len(s['vps']) for s in scenes)} views",
            "object_views": ov, "batched_ms": batched_ms, "plain_ms": plain_ms,
            "batched_object_views_per_s": ov / (batched_ms / 1e3), "plain_object_views_per_s": ov / (plain_ms / 1e3),
            "batched_vs_plain": plain_ms / batched_ms, "tuning": tuning,
            "plain_launches_per_step": sum(len(s["vps"]) for s in scenes)}


# ---- serving (config 4) ----------------------------------------------------------------------------
def run_serving(ctx, args) -> dict:
    """64 Poisson clients (mean args.serve_rate requests/s) against a catalogue whose
    resident bytes exceed the HBM budget (LRU eviction runs); p50/p99 latency from the
    scheduled arrival to the completion seen by the server."""
    from pipeline_gb300 import native, serving

    budget = int(args.serve_budget_gb * 1e9)
    templates = serving.make_templates(seed=4, n_templates=args.serve_templates)
    avg = float(np.mean([serving.scene_bytes(t["n"], t["mats"].shape[0]) for t in templates]))
    n_scenes = int(math.ceil(1.25 * budget / avg))
    times, scenes, nviews, vps = serving.schedule(seed=44, n_scenes=n_scenes,
                                                  duration_s=args.serve_seconds, rate=args.serve_rate)
    with native.Server(ctx, budget, n_streams=3, max_batch_objects=48 << 20) as srv:
        for k in range(n_scenes):
            t = templates[k % len(templates)]
            srv.add_scene(k, t["lower"], t["extent"], t["xform"], t["mats"])
        res = serving.run_load(srv, times, scenes, nviews, vps, warmup_s=args.serve_warmup)
        st = srv.stats()
    res.update({"budget_gb": budget / 1e9, "catalogue_scenes": n_scenes,
                "catalogue_gb": n_scenes * avg / 1e9, "templates": len(templates),
                "clients": 64, "rate_req_per_s": args.serve_rate, "seconds": args.serve_seconds,
                "warmup_s": args.serve_warmup, "evictions": st["scene_evictions"],
                "uploads": st["scene_uploads"], "upload_gb": st["upload_bytes"] / 1e9,
                "batches": st["batches"], "max_batch_requests": st["max_batch_requests"],
                "streams": 3, "scheduler": {k: st[k] for k in ("max_turn_us", "slow_turns",
                                                               "max_upload_call_us", "max_evict_call_us",
                                                               "reserved_bytes")}})
    return res


# ---- CPU baseline (oracle port on the host cores) ----------------------------------------------
def cpu_baseline(wl, sample: int, threads: int, reps: int = 3) -> dict:
    import oracle

    sc = wl.sc
    m = min(sample, wl.n)
    obbs = oracle.build_obbs(sc["lower"][:, :m], sc["extent"][:, :m], sc["xform"][:m], sc["mats"])
    prev = [np.zeros((m + 31) // 32, np.uint32) for _ in range(wl.v)]
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        for v in range(wl.v):
            bits = oracle.cull_obbs(obbs, sc["vps"][v], threads=threads)
            oracle.update_changed(prev[v], bits, m)
        ts.append(time.perf_counter() - t0)
    t_warm = statistics.median(ts)
    t0 = time.perf_counter()
    oracle.build_obbs(sc["lower"][:, :m], sc["extent"][:, :m], sc["xform"][:m], sc["mats"])
    t_obb = time.perf_counter() - t0
    return {"value": m * wl.v / t_warm, "unit": "object-views/s", "cores": threads, "kind": "port",
            "sample": f"first {m} objects x {wl.v} views, OBB cache warm, median of {reps}",
            "cold_value": m * wl.v / (t_warm + t_obb)}


def run_reference(args, dist: Dist) -> dict | None:
    """The reference CPU culling path (the oracle port of cpu::ManagerImpl::cull over the
    cached OBBs + ResultBitSet::updateChanged, dp/culling/cpu/src/ManagerImpl.cpp:467-518,
    dp/culling/src/ResultBitSet.cpp:61-108) on all host cores, on the same workload as our
    arm: the whole scene (N x objects per GPU, on rank 0 alone), the same 8 views and the
    same camera path.  The OBBs are built once (the reference's cache, GroupCPU::updateOBBs,
    cpu/src/ManagerImpl.cpp:114-162) before the timed steps; a cold step (every matrix
    changed) adds one OBB rebuild, timed separately."""
    if dist.rank != 0:
        return None
    import oracle

    oracle.build(with_reference=False)
    threads = os.cpu_count() or 1
    wl = Stress(seed=3, n=args.objects, t=args.transforms, world=dist.world, end=args.objects * dist.world)
    sc = wl.sc
    m = wl.n
    t0 = time.perf_counter()
    obbs = oracle.build_obbs(sc["lower"], sc["extent"], sc["xform"], sc["mats"])
    t_obb = time.perf_counter() - t0
    prev = [np.zeros((m + 31) // 32, np.uint32) for _ in range(wl.v)]
    rng = np.random.default_rng(17)
    frames = make_frames(rng, sc["vps"], args.warmup + args.steps)
    ts = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for v in range(wl.v):
            bits = oracle.cull_obbs(obbs, frames[i][v], threads=threads)
            oracle.update_changed(prev[v], bits, m)
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    t = sum(ts) / len(ts)
    value = m * wl.v / t
    desc = (f"all {m} objects x {wl.v} views per step, OBB cache warm (built once, {t_obb * 1e3:.0f} ms on 1 thread, "
            f"as the reference builds it), cull on {threads} threads")
    return {"impl": "reference", "metric": METRIC,
            "value": value, "unit": "object-views/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; the reference publishes no dataset)",
            "config": {"workload": wl.describe, "objects_per_gpu": args.objects, "objects_total": m,
                       "transforms": wl.t, "views": wl.v, "same_config": True,
                       "camera": "the same jittered camera path as our arm (seed 17)"},
            "cold": {"value": m * wl.v / (t + t_obb), "unit": "object-views/s", "ms_per_step": (t + t_obb) * 1e3,
                     "obb_rebuild_ms": t_obb * 1e3,
                     "note": "a step after every matrix changed: one OBB rebuild (single thread, as "
                             "GroupCPU::updateOBBs) plus the warm cull"},
            "cpu_baseline": {"value": value, "unit": "object-views/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "object-views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="stress", choices=["stress", "serving", "plain", "hierarchy", "batched"])
    ap.add_argument("--tuning", default=None, help="JSON tuning (default: autotuner)")
    ap.add_argument("--cpu-sample", type=int, default=1_000_000)
    ap.add_argument("--objects", type=int, default=STRESS_N, help="objects per GPU (smaller cases for profiling)")
    ap.add_argument("--transforms", type=int, default=STRESS_T)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="serving run length (0 = skip)")
    ap.add_argument("--serve-warmup", type=float, default=1.0)
    ap.add_argument("--serve-rate", type=float, default=20_000.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-templates", type=int, default=32)
    ap.add_argument("--exact-only", action="store_true",
                    help="disable the conservative prefilter (ablation; results are identical)")
    ap.add_argument("--no-box-cache", action="store_true",
                    help="disable the groups' box cache (every launch transforms every box)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the plain, hierarchy and batched configurations on the default line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist = Dist(args.gpus)
    if args.impl == "reference":
        out = run_reference(args, dist)
    elif args.workload in ("serving", "plain", "hierarchy", "batched"):
        from pipeline_gb300 import build, native

        build.build_all()
        ctx = native.Context(dist.local)
        fn = {"serving": run_serving, "plain": run_plain_config, "hierarchy": run_hierarchy_config,
              "batched": run_batched_config}[args.workload]
        out = {"workload": args.workload, "result": fn(ctx, args)}
        ctx.close()
    else:
        out = run_ours(args, dist)
        if out is not None and dist.rank == 0 and not args.no_cpu_baseline:
            wl_cpu = Stress(seed=3, n=args.objects, t=args.transforms, end=args.cpu_sample)
            out["cpu_baseline"] = cpu_baseline(wl_cpu, args.cpu_sample, 1)
            out["cpu_baseline"]["all_cores"] = cpu_baseline(wl_cpu, args.cpu_sample, os.cpu_count() or 1, reps=3)
    if out is not None and dist.rank == 0:
        print(json.dumps(out))
    dist.close()


if __name__ == "__main__":
    main()
