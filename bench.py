"""Benchmark of the visual-hull path: hulls/s on the level-9, 32x1024^2 partial-view workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--mode headline|hetero|serve]

Headline workload (one "step"): the visual hulls of Q requests (default 4),
each a distinct seeded scene of 8 ellipsoids + 20 thin capsules seen by 32
cameras at radius 1.4 (fov 50 deg, OpenGL convention) as float32 masks
[32,1024,1024,1], masks_partial=True, level 9, unique vertices.  The masks are
synthetic (ray tests at pixel centres) and stand in for the reference's
OpenGL-rendered dataset.  Each request's masks are 128 MiB, so the inputs
exceed L2 between timed iterations.

GB300 arm: inputs resident in HBM.  `value` is hulls/s of the batched form
(all Q requests of a step in one th_visual_hull_batch call: one persistent
carve launch over the Q octrees).  Beside it: the plain drop-in
(torchhull_gb300.visual_hull, one request per call) as hulls/s and p50/p99
per hull (as a caller runs it: the pipeline replayed as a CUDA graph), stage
times from a separate profiled pass, whose CUDA events between the stages
disable the replay (the largest stage is the roofline line), and `e2e`: the
plain drop-in fed from pinned host memory, every request's masks and
transforms copied in and its mesh copied back inside the timed region, the
copies overlapped with the neighbouring hulls on one side stream (the
previous mesh out, then the next request in; `e2e_batched`: the batched
step with the same copies, overlapped the same way).
Under torchrun every rank serves its own requests (weak scaling, no
collective on the data path).

--mode hetero: 64 heterogeneous requests (views U{4..48}, side
U{256,512,768,1024}, level U{6..9}, partial ~ Bernoulli(0.3)), batched vs plain.
--mode blur: the blur configuration (24 OpenCV views of 512^2, blur k=9 sigma=2,
level 8) as one fused request against blur and hull as two calls.
--mode mc: torchhull.marching_cubes on the reference benchmark's sphere SDF
volumes (100^3 .. 600^3, dense and sparse), ms per call.
--mode serve: Poisson arrivals (default 200/s for 20 s) from a pool of
pregenerated requests of the heterogeneous distribution plus 2 % large ones
(64 views of 2048^2, level 10) through the continuous-batching server (60 GB
admission budget), against the same stream served one request at a time.

Also in the headline line (one GPU): `reference_cuda`, torchhull's own CUDA
extension built from its unmodified sources (oracle/ref_build.py) timed on the
same requests, one per call, as the comparison point of the plain drop-in;
`cfg1` (8 views of 256^2, level 6) and `cfg2` (the blur configuration, fused
and as two calls, and the reference's two calls); `hetero64` (the 64-request
mix, batched against plain); `serve` (Poisson arrivals at 200/s for 20 s with
2 % large requests, host inputs copied in inside the latency, continuous
batching against one request at a time).

Reference arm (--impl reference): the reference has no CPU path, so it times
the CPU restatement of the reference's algorithm (oracle/) with all host
threads.  One step is one octant of the cube at the same leaf size (level 8
over half the cube length): 8 steps cover one hull.  The GB300 arm's
`cpu_baseline` times the same 8 octants.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# CUDA maps streams onto a few hardware work queues (8 by default), and streams
# that share one can wait on each other's work.  This process runs the
# library's own streams, the serving slots' and the copy stream of the
# end-to-end legs beside the hulls' stream: give them 32 queues.  Must be set
# before CUDA initialises.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

LEVEL = 9
VIEWS = 32
SIDE = 1024
METRIC = "hulls/s, level 9, 32x1024^2 views, partial masks (batched form; plain p50/p99 ms per hull alongside)"
WORKLOAD = ("partial-view visual hull: 32 views of 1024x1024 float32 masks, level 9, masks_partial=True, "
            "unique_verts=True, OpenGL, 8 ellipsoids + 20 capsules")
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
# DRAM bytes (read + write) per launch of a stage's dominant kernel, from one ncu capture of the
# same workload's first request (not measured by this run): dram__bytes_read.sum +
# dram__bytes_write.sum of the level-8 classify_items_kernel launch.
NCU_TRAFFIC = {"carve_level_8": 60.8e6}
NCU_TRAFFIC_SOURCE = ("ncu --set full capture of classify_items_kernel, level 8, first request of this workload "
                      "(dram__bytes_read.sum + dram__bytes_write.sum); a separate capture, not this run")


def peaks() -> tuple[float, str]:
    try:
        d = json.loads(MEASURED_PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == len(self.FIELDS):
                self.samples.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=5)
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for s in self.samples:
            for name, v in zip(names, s[2:], strict=True):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def algorithmic_bytes(info_levels: list[int], corners: int, verts: int, faces: int, B: int, H: int, W: int,
                      mask_bytes: int, carve_items: list | None = None, field_items: float | None = None) -> dict:
    """Per-stage algorithmic bytes of one hull (the formula of the design notes), over the units the
    kernels evaluate: carve_items (parent, view) items per level, 8 children x 16 bytes of
    integral-image reads each, and field_items (corner, view) samples of 16 bytes; views that the
    inherited skip and out-of-frame masks leave out are read by no kernel and not counted.  Without
    the counts every pair is counted, as the reference evaluates them."""
    out = {"integral_image": (mask_bytes + 4) * B * H * W}
    carve = []
    for i in range(len(info_levels) - 1):
        p, pn = info_levels[i], info_levels[i + 1]
        items = carve_items[i] if carve_items is not None else p * B
        carve.append(8 * p + 8 * items * 16 + 8 * pn)
    out["carve"] = carve
    leaves = info_levels[-1]
    out["corners"] = 8 * 8 * leaves + 8 * corners
    pairs = field_items if field_items is not None else corners * B
    out["field"] = pairs * 16 + 4 * corners + 8 * corners
    out["marching_cubes"] = corners * (16 + 8 * 16) + 12 * verts + 24 * faces
    return out


def as_tuple(r):
    return (r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
            r.transforms_convention, r.unique_verts)


def percentile(sorted_vals: list[float], p: float) -> float | None:
    if not sorted_vals:
        return None
    return sorted_vals[min(len(sorted_vals) - 1, int(round(p / 100.0 * (len(sorted_vals) - 1))))]


def replica_seeds(rank: int, count: int, base: int = 3) -> list[int]:
    """Seeds of a rank's own requests: every rank serves different scenes (replicas, weak scaling)."""
    return [base + 1000 * rank + q for q in range(count)]


def whole_job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Units of all ranks per second of the slowest rank (the job ends when the last rank does)."""
    return units_per_rank * world / seconds_max


def max_over_ranks(x: float, world: int, dev) -> float:
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], device=dev, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def timed_batches(th, tuples, steps: int, dev, world: int) -> float:
    """Device time (ms, max over ranks) of `steps` batched calls."""
    import torch
    import torch.distributed as dist

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        th._C.visual_hull_batch(tuples)
    stop.record()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    return max_over_ranks(start.elapsed_time(stop), world, dev)


def timed_plain(th, reqs, steps: int, dev, world: int, local: int, profile: bool):
    """Plain drop-in, one request per call: (ms max over ranks, per-hull ms, stage times)."""
    import torch
    import torch.distributed as dist

    if profile:
        th._C.set_profiling(local, True)
    per_hull: list[float] = []
    stages: dict[str, list] = {}
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        for r in reqs:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            th.visual_hull(**r.kwargs())
            e1.record()
            e1.synchronize()
            per_hull.append(e0.elapsed_time(e1))
            if profile:
                for k, val in th._C.stage_times(local).items():
                    stages.setdefault(k, []).append(val)
    stop.record()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    if profile:
        th._C.set_profiling(local, False)
    return max_over_ranks(start.elapsed_time(stop), world, dev), sorted(per_hull), stages


def host_copy(th, method: str):
    """The copy the end-to-end legs move their bytes with, on the current stream: "sm" is
    torchhull_gb300's copy kernel (th_copy: a few blocks of SMs over the pinned buffers' device
    mappings), "dma" is cudaMemcpyAsync (a copy engine).  With copy-engine copies overlapping the
    hulls, about one loop of three on GB300 lost ~70-80 ms: a few consecutive copies ran at a
    tenth of their rate (raw cudaMemcpyAsync as well as torch's copies, either direction).  Plain hulls: the copy kernel showed no
    stall in 40 loops and ran ~5% below the stall-free copy-engine loops.  Batched hulls: its few
    blocks find little room beside the persistent carve kernel (~232 against ~342 hulls/s for
    stall-free copy-engine loops), so that leg keeps the copy engines."""
    if method == "sm":
        return th._C.copy_on_sms

    def dma(dst, src):
        dst.copy_(src, non_blocking=True)

    return dma


def e2e_plain_pipelined(th, reqs, steps: int, dev, world: int, copy: str = "sm") -> tuple[float, int, int, dict]:
    """End to end through the plain drop-in (torchhull_gb300.visual_hull) from
    pinned host memory: hull i runs on the compute stream while one copy stream
    first copies hull i-1's mesh out to pinned host memory and then request
    i+1's masks and transforms in (two device slots).  Every copy of every step
    is inside the timed region; copy names the copy method (host_copy).
    Returns (hulls/s, h2d bytes per step, d2h bytes per step, allocator
    counters of the timed loop).

    The two directions share one stream, so one copy at a time runs beside a
    hull (per hull 134 MB in at ~130 GB/s and ~211 MB out at ~190 GB/s with
    the copy kernel: ~2.2 ms, inside the ~3.1 ms hull)."""
    import torch
    import torch.distributed as dist

    xfer = host_copy(th, copy)
    Q = len(reqs)
    shape, tshape = reqs[0].masks.shape, reqs[0].transforms.shape
    assert all(r.masks.shape == shape and r.transforms.shape == tshape for r in reqs)
    host_in = [(r.masks.cpu().pin_memory(), r.transforms.cpu().pin_memory()) for r in reqs]
    slots = [(torch.empty_like(reqs[0].masks), torch.empty_like(reqs[0].transforms)) for _ in range(2)]
    # the meshes are deterministic: pinned result buffers sized from one untimed call each
    host_out = []
    for r in reqs:
        v, f = th.visual_hull(**r.kwargs())
        host_out.append((torch.empty(v.shape, dtype=v.dtype, pin_memory=True),
                         torch.empty(f.shape, dtype=f.dtype, pin_memory=True)))
    h2d = sum(m.numel() * m.element_size() + t.numel() * t.element_size() for m, t in host_in)
    d2h = sum(v.numel() * v.element_size() + f.numel() * f.element_size() for v, f in host_out)

    comp = torch.cuda.current_stream(dev)
    copies = torch.cuda.Stream(dev)
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]
    order = [q for _ in range(steps) for q in range(Q)]

    def copy_in(order, i):
        s = i % 2
        with torch.cuda.stream(copies):
            copies.wait_event(free[s])  # hull i-2 is done with slot s
            xfer(slots[s][0], host_in[order[i]][0])
            xfer(slots[s][1], host_in[order[i]][1])
            ready[s].record(copies)

    def run(order):
        for i in range(min(2, len(order))):
            copy_in(order, i)
        for i, q in enumerate(order):
            s = i % 2
            comp.wait_event(ready[s])
            kw = reqs[q].kwargs()
            kw["masks"], kw["transforms"] = slots[s]
            v, f = th.visual_hull(**kw)
            free[s].record(comp)
            done = torch.cuda.Event()
            done.record(comp)
            # on the copy stream: hull i's mesh out, then request i+2's inputs in
            # (into the slot hull i has just released); both overlap hull i+1
            with torch.cuda.stream(copies):
                copies.wait_event(done)
                xfer(host_out[q][0], v)
                xfer(host_out[q][1], f)
                v.record_stream(copies)
                f.record_stream(copies)
            if i + 2 < len(order):
                copy_in(order, i + 2)
        torch.cuda.synchronize()

    # one untimed pass of the same loop: the caching allocator settles on the
    # blocks this pattern of allocations and cross-stream frees needs
    run(list(range(Q)))
    stats0 = torch.cuda.memory_stats(dev)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run(order)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    stats1 = torch.cuda.memory_stats(dev)
    allocator = {k: stats1.get(k, 0) - stats0.get(k, 0)
                 for k in ("segment.all.allocated", "segment.all.freed", "num_alloc_retries")}
    return Q * steps * world / e2e_s, h2d, d2h, allocator


def copy_bandwidth(reqs, dev, reps: int = 3) -> dict:
    """Pinned host <-> device copy bandwidth of one request's masks, measured alone with CUDA events
    (best of reps).  The end-to-end legs move these bytes every hull, so their result depends on
    this bandwidth, which varies on a shared machine; it is reported beside them."""
    import torch

    src = reqs[0].masks
    host = torch.empty(src.shape, dtype=src.dtype, pin_memory=True)
    dst = torch.empty_like(src)
    nbytes = src.numel() * src.element_size()
    out = {}
    for name, fn in (("h2d", lambda: dst.copy_(host, non_blocking=True)),
                     ("d2h", lambda: host.copy_(src, non_blocking=True))):
        best = float("inf")
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[f"{name}_gbs"] = nbytes / (best / 1000.0) / 1e9
    out["bytes"] = nbytes
    return out


def run_gb300(args) -> dict | None:
    import torch
    import torch.distributed as dist

    import torchhull_gb300 as th
    from torchhull_gb300 import scenes

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    th._C.set_carve_kernel(local, {"auto": 0, "views": 1, "items": 2}[args.carve_kernel])
    th._C.set_batch_route(local, args.batch_route == "on")
    th._C.set_field_ones(local, args.field_ones == "on")
    th._C.set_field_masks(local, args.field_masks == "on")

    if args.mode == "hetero":
        return finish(run_hetero(args, th, scenes, dev, world, rank), world)
    if args.mode == "serve":
        return finish(run_serve(args, th, scenes, dev, world, rank), world)
    if args.mode == "mc":
        return finish(run_mc(args, th, dev, world, rank), world)
    if args.mode == "blur":
        return finish(run_blur(args, th, scenes, dev, world, rank), world)

    Q = args.requests
    reqs = [scenes.partial_request(device=dev, seed=seed) for seed in replica_seeds(rank, Q)]
    tuples = [as_tuple(r) for r in reqs]
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        th._C.visual_hull_batch(tuples)
        for r in reqs:
            th.visual_hull(**r.kwargs())
    torch.cuda.synchronize()

    # batched form: the value
    sampler = ClockSampler(local)
    launches0 = th._C.launch_count()
    sampler.start()
    batch_ms = timed_batches(th, tuples, args.steps, dev, world)
    clocks = sampler.stop()
    launches = th._C.launch_count() - launches0
    value = whole_job_rate(Q * args.steps, world, batch_ms / 1000.0)

    # plain drop-in: throughput and latency as a caller sees them (stage events
    # off, so the pipeline is replayed as a CUDA graph), then stage times from
    # a separate profiled pass (events between the stages, direct launches)
    plain_ms, per_hull, _ = timed_plain(th, reqs, args.steps, dev, world, local, profile=False)
    plain_value = Q * args.steps * world / (plain_ms / 1000.0)
    _, per_hull_profiled, stages = timed_plain(th, reqs, max(1, args.steps // 2), dev, world, local, profile=True)

    # end to end through the plain drop-in, copies pipelined against the hulls
    e2e_steps = args.steps
    copy_gbs = copy_bandwidth(reqs, dev)
    e2e_value, h2d, d2h, e2e_alloc = e2e_plain_pipelined(th, reqs, e2e_steps, dev, world, copy=args.e2e_copy)
    # the same loop once with the other copy method, for comparison
    other_copy = "dma" if args.e2e_copy == "sm" else "sm"
    e2e_other = e2e_plain_pipelined(th, reqs, e2e_steps, dev, world, copy=other_copy)[0]

    # end to end through the batched form: while step k's batch runs, one side
    # stream copies step k-1's meshes out and then step k+1's inputs in (two
    # device slots), as for the plain drop-in
    host_masks = [r.masks.cpu().pin_memory() for r in reqs]
    host_tf = [r.transforms.cpu().pin_memory() for r in reqs]
    slots = [[(torch.empty_like(r.masks), torch.empty_like(r.transforms)) for r in reqs] for _ in range(2)]
    first = th._C.visual_hull_batch(tuples)
    host_out = [(torch.empty(v.shape, dtype=v.dtype, pin_memory=True),
                 torch.empty(f.shape, dtype=f.dtype, pin_memory=True)) for v, f in first]
    comp = torch.cuda.current_stream(dev)
    copies = torch.cuda.Stream(dev)
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]
    xfer = host_copy(th, args.e2e_batched_copy)

    def batch_in(k):
        s = k % 2
        with torch.cuda.stream(copies):
            copies.wait_event(free[s])  # step k-2 is done with slot s
            for q in range(Q):
                xfer(slots[s][q][0], host_masks[q])
                xfer(slots[s][q][1], host_tf[q])
            ready[s].record(copies)

    def run_batches(steps):
        for k in range(min(2, steps)):
            batch_in(k)
        for k in range(steps):
            s = k % 2
            comp.wait_event(ready[s])
            out = th._C.visual_hull_batch([slots[s][q] + tuples[q][2:] for q in range(Q)])
            free[s].record(comp)
            done = torch.cuda.Event()
            done.record(comp)
            with torch.cuda.stream(copies):
                copies.wait_event(done)
                for (v, f), (vh, fh) in zip(out, host_out, strict=True):
                    xfer(vh, v)
                    xfer(fh, f)
                    v.record_stream(copies)
                    f.record_stream(copies)
            if k + 2 < steps:
                batch_in(k + 2)
        torch.cuda.synchronize()

    run_batches(2)  # untimed: the allocator settles on this loop's blocks
    bstats0 = torch.cuda.memory_stats(dev)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_batches(e2e_steps)
    e2e_batched = Q * e2e_steps * world / max_over_ranks(time.perf_counter() - t0, world, dev)
    bstats1 = torch.cuda.memory_stats(dev)
    e2e_batched_alloc = {k: bstats1.get(k, 0) - bstats0.get(k, 0)
                         for k in ("segment.all.allocated", "segment.all.freed", "num_alloc_retries")}
    del slots, host_out, first

    # the other configurations and the reference's CUDA build, measured after the timed region
    # (one GPU only: under torchrun every rank times the headline alone)
    extras = {}
    if world == 1 and not args.no_extras:
        extras = headline_extras(args, th, scenes, dev, world, rank, reqs, plain_value)

    if rank != 0:
        return finish(None, world)

    # roofline of the dominant stage, from the stage events of the plain timed region
    r0 = reqs[0]
    info = th.visual_hull_with_candidate_voxels(**r0.kwargs())
    levels = [c.numel() for c in info[2]]
    field = th.sparse_visual_hull_field(r0.masks, r0.transforms, LEVEL, r0.cube_corner_bfl, r0.cube_length, True,
                                        "opengl")
    corners = field.values().numel()
    nv, nf = info[0].shape[0], info[1].shape[0]
    mean = {k: (statistics.fmean(v) if not isinstance(v[0], list) else [statistics.fmean(x) for x in zip(*v)])
            for k, v in stages.items()}
    algo = algorithmic_bytes(levels, corners, nv, nf, VIEWS, SIDE, SIDE, 4, mean.get("carve_items"),
                             mean.get("field_items"))
    every_pair = algorithmic_bytes(levels, corners, nv, nf, VIEWS, SIDE, SIDE, 4)
    cands = [("integral_image", "sat_columns_kernel+sat_rows_kernel", mean["integral_image"], algo["integral_image"],
              every_pair["integral_image"])]
    for i, ms in enumerate(mean["carve"]):
        cands.append((f"carve_level_{i}", "classify_*_kernel+scan", ms, algo["carve"][i], every_pair["carve"][i]))
    cands += [("corners", "mark_corners_kernel+scans", mean["corners"], algo["corners"], every_pair["corners"]),
              ("field", "ones_kernel+field_masked_kernel", mean["field"], algo["field"], every_pair["field"]),
              ("marching_cubes", "mc_cells_kernel+scan", mean["marching_cubes"], algo["marching_cubes"],
               every_pair["marching_cubes"])]
    dom = max(cands, key=lambda c: c[2])
    peak, peak_kind = peaks()
    achieved = dom[3] / (dom[2] / 1000.0) / 1e9
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "hulls/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": batch_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: seeded ray-ellipsoid/capsule masks (stand-in for the reference's rendered dataset)",
        "config": {"workload": WORKLOAD, "requests_per_step": Q, "level": LEVEL, "views": VIEWS, "side": SIDE,
                   "l2": "inputs larger than L2 (128 MiB of masks + 128 MiB SAT per request)",
                   "path": "batched form (th_visual_hull_batch: one persistent carve launch per step)",
                   "field_ones": args.field_ones, "field_masks": args.field_masks,
                   "mesh_verts": nv, "mesh_faces": nf, "leaves": levels[-1], "corners": corners},
        "plain": {"value": plain_value, "unit": "hulls/s", "p50_ms": percentile(per_hull, 50),
                  "p99_ms": percentile(per_hull, 99), "path": "torchhull_gb300.visual_hull, one request per call",
                  "profiled_p50_ms": percentile(per_hull_profiled, 50)},
        "batched_over_plain": value / plain_value,
        "p50_ms": percentile(per_hull, 50),
        "p99_ms": percentile(per_hull, 99),
        "stage_ms": {k: v for k, v in mean.items() if not k.endswith("_items")},
        "stage_units": {"carve_items": mean.get("carve_items"), "field_items": mean.get("field_items"),
                        "every_carve_pair": [lv * VIEWS for lv in levels[:-1]], "every_field_pair": corners * VIEWS},
        "e2e": {"value": e2e_value, "unit": "hulls/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "torchhull_gb300.visual_hull from pinned host memory; on one side stream the "
                        "previous mesh out, then the next request in, overlapping the hull",
                "copy_method": args.e2e_copy, f"value_with_{other_copy}_copies": e2e_other,
                "copy_bandwidth": copy_gbs, "allocator_in_timed_loop": e2e_alloc},
        "e2e_batched": {"value": e2e_batched, "unit": "hulls/s",
                        "path": "th_visual_hull_batch per step; on one side stream the previous step's meshes out, "
                                "then the next step's inputs in, overlapping the batch",
                        "copy_method": args.e2e_batched_copy, "allocator_in_timed_loop": e2e_batched_alloc},
        "roofline": {"bound": "hbm", "kernel": dom[1], "stage": dom[0], "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": dom[3], "ms": dom[2], "traffic": NCU_TRAFFIC.get(dom[0]),
                     "traffic_source": NCU_TRAFFIC_SOURCE if dom[0] in NCU_TRAFFIC else None,
                     "every_pair_bytes": dom[4],
                     "note": "bytes of the units the kernels evaluate; every_pair_bytes counts every (cell, view) "
                             "or (corner, view) pair, as the reference evaluates them"},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    line.update(extras)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(reqs[0], samples=args.cpu_samples)
    return finish(line, world)


def finish(line, world):
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return line


def hetero_measure(args, th, scenes, dev, world, rank) -> dict:
    """64 heterogeneous requests: one batched call per step against the plain drop-in, one call per request."""
    import torch

    reqs = scenes.batched_requests(count=args.hetero_count, seed=4 + 1000 * rank, device=dev)
    tuples = [as_tuple(r) for r in reqs]
    for _ in range(max(1, args.warmup)):
        th._C.visual_hull_batch(tuples)
        for r in reqs:
            th.visual_hull(**r.kwargs())
    torch.cuda.synchronize()
    steps = max(1, args.hetero_steps)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    launches0 = th._C.launch_count()
    batch_ms = timed_batches(th, tuples, steps, dev, world)
    launches = th._C.launch_count() - launches0
    clocks = sampler.stop()
    plain_ms, per_hull, _ = timed_plain(th, reqs, steps, dev, world, dev.index or 0, profile=False)
    n = len(reqs)
    value = n * steps * world / (batch_ms / 1000.0)
    plain_value = n * steps * world / (plain_ms / 1000.0)
    return {"value": value, "unit": "hulls/s", "steps": steps, "ms_per_step": batch_ms / steps,
            "requests_per_step": n,
            "workload": f"{n} requests: views U{{4..48}}, side U{{256,512,768,1024}}, level U{{6..9}}, "
                        "masks_partial ~ Bernoulli(0.3), float32, inputs resident",
            "plain": {"value": plain_value, "unit": "hulls/s", "p50_ms": percentile(per_hull, 50),
                      "p99_ms": percentile(per_hull, 99)},
            "batched_over_plain": value / plain_value, "clocks": clocks, "gpu_launches": launches}


def run_hetero(args, th, scenes, dev, world, rank):
    m = hetero_measure(args, th, scenes, dev, world, rank)
    if rank != 0:
        return None
    return {
        "metric": "hulls/s, 64 heterogeneous requests (batched form)", "value": m["value"], "unit": "hulls/s",
        "n_gpus": world, "steps": m["steps"], "warmup": args.warmup, "ms_per_step": m["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded ray-ellipsoid/capsule masks",
        "config": {"workload": m["workload"], "requests_per_step": m["requests_per_step"]},
        "plain": m["plain"], "batched_over_plain": m["batched_over_plain"],
        "clocks": m["clocks"], "gpu_launches": m["gpu_launches"],
    }


def sphere_sdf(size: int, dev):
    """The reference benchmark's volume (benchmarks/test_bench_marching_cubes.py:68-86)."""
    import torch

    g = torch.arange(size, device=dev)
    pts = torch.stack(torch.meshgrid(3 * [g], indexing="ij"), dim=0).reshape(3, -1).T.to(torch.float32)
    center = torch.full((3,), size / 2, dtype=torch.float32, device=dev)
    radius = 0.8731945 * (size / 2)
    return (torch.linalg.norm(pts - center[None], dim=1) - radius).reshape(1, size, size, size)


def run_mc(args, th, dev, world, rank):
    """Marching cubes on the reference benchmark's sphere volumes, dense and sparse (truncation 2)."""
    import torch

    rows = []
    for size in [int(x) for x in args.mc_sizes.split(",")]:
        dense = sphere_sdf(size, dev)
        sparse_src = dense.clone()
        sparse_src[sparse_src.abs() > 2] = 0
        sparse = sparse_src.to_sparse()
        del sparse_src
        for kind, vol in (("dense", dense), ("sparse", sparse)):
            for _ in range(max(3, args.warmup)):
                v, f = th.marching_cubes(vol, 0.0, False)
            torch.cuda.synchronize()
            times = []
            for _ in range(args.steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                th.marching_cubes(vol, 0.0, False)
                e1.record()
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            times.sort()
            nbytes = dense.numel() * 4 if kind == "dense" else vol.values().numel() * (4 + 32)
            rows.append({"size": size, "kind": kind, "p50_ms": percentile(times, 50), "min_ms": times[0],
                         "verts": int(v.shape[0]), "faces": int(f.shape[0]), "input_bytes": nbytes,
                         "input_gbs": nbytes / (percentile(times, 50) / 1000.0) / 1e9})
        del dense, sparse
        torch.cuda.empty_cache()
    if rank != 0:
        return None
    head = max((r for r in rows if r["kind"] == "dense"), key=lambda r: r["size"])
    return {"metric": "marching_cubes ms per call, largest dense float32 sphere SDF (reference benchmark volumes)",
            "value": head["p50_ms"], "unit": "ms", "size": head["size"], "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["p50_ms"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic: sphere SDF of benchmarks/test_bench_marching_cubes.py",
            "config": {"workload": "torchhull.marching_cubes(sdf, isolevel=0, return_local_coords=False), sizes "
                                   "100..600, dense and sparse (|sdf| <= 2)"},
            "table": rows}


def run_blur(args, th, scenes, dev, world, rank):
    """The blur configuration: 5 ellipsoids, 24 OpenCV views of 512^2, blur k=9 sigma=2, then level 8."""
    import torch

    r = scenes.blur_request(device=dev, seed=2 + 1000 * rank)
    hull_args = (r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial, r.transforms_convention)

    def two_calls():
        return th.visual_hull(th.gaussian_blur(r.masks, 9, 2.0), *hull_args)

    def fused():
        return th.visual_hull_blurred(r.masks, *hull_args, 9, 2.0)

    out = {}
    for name, fn in (("fused", fused), ("two_calls", two_calls)):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        e1.synchronize()
        out[name] = max_over_ranks(e0.elapsed_time(e1), world, dev) / args.steps
    if rank != 0:
        return None
    return {"metric": "hulls/s, blur k=9 sigma=2 then level-8 hull, 24x512^2 OpenCV views (fused request)",
            "value": 1000.0 * world / out["fused"], "unit": "hulls/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["fused"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded ray-ellipsoid masks",
            "config": {"workload": "5 ellipsoids, 24 OpenCV views of 512x512 float32, gaussian_blur(k=9, sigma=2, "
                                   "sparse), visual_hull level 8, full masks"},
            "two_calls_ms": out["two_calls"], "fused_over_two_calls": out["two_calls"] / out["fused"]}


def serve_measure(args, th, scenes, dev, world, rank, policies=("none", "large_first", "exclusive_large")) -> dict:
    """Poisson arrivals from a pool of pregenerated requests of the heterogeneous distribution plus 2 %
    large ones (64 x 2048^2, level 10), their masks and transforms in pinned host memory: each request
    is copied in by the server inside its measured latency (arrival -> result on the device).  The
    continuous-batching server against the same stream served one request at a time."""
    import numpy as np
    import torch

    from torchhull_gb300.serve import HullServer

    def to_host(r):
        return scenes.HullRequest(r.masks.cpu().pin_memory(), r.transforms.cpu().pin_memory(), r.level,
                                  r.cube_corner_bfl, r.cube_length, r.masks_partial, r.transforms_convention,
                                  r.unique_verts)

    pool_dev = scenes.batched_requests(count=args.serve_pool, seed=6 + 1000 * rank, device=dev)
    large_dev = [scenes.make_request(9000 + 1000 * rank + i, 64, 2048, 10, False, device=dev)
                 for i in range(args.serve_large)]
    for r in pool_dev + large_dev:  # warm the autotuner and the allocator
        th.visual_hull(**r.kwargs())
    torch.cuda.synchronize()
    pool = [to_host(r) for r in pool_dev]
    large = [to_host(r) for r in large_dev]
    del pool_dev, large_dev
    torch.cuda.empty_cache()
    rng = np.random.default_rng(7 + rank)
    n = int(args.rate * args.duration)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=n))
    picks = [large[i % len(large)] if (large and rng.random() < 0.02) else pool[int(rng.integers(len(pool)))]
             for i in range(n)]

    def serve(slots, priority="none", max_batch=1, burst=0):
        """burst > 0: that many requests from the pool submitted at once (capacity), else the arrivals."""
        with HullServer(device=dev.index or 0, slots=slots, budget_bytes=60e9, priority=priority,
                        max_batch=max_batch) as server:
            # every slot's context: pools sized, carve kernel tuned, graphs captured for the pool's shapes
            server.warm_up(pool + large[:1])
            server.latencies_ms.clear()
            server.queue_ms.clear()
            t0 = time.perf_counter()
            futures = []
            if burst:
                futures = [server.submit(pool[i % len(pool)]) for i in range(burst)]
            else:
                for t, r in zip(arrivals, picks, strict=True):
                    delay = t - (time.perf_counter() - t0)
                    if delay > 0:
                        time.sleep(delay)
                    futures.append(server.submit(r))
            for f in futures:
                f.result(timeout=600)  # a failed server raises here instead of hanging the run
            wall = time.perf_counter() - t0
            st = server.stats()
            count = burst or n
            return {"value": count / wall, "unit": "hulls/s", "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                    "mean_queue_ms": st["mean_queue_ms"], "wall_s": wall}

    out = {p: serve(args.serve_slots, p) for p in policies}
    out["batched"] = serve(args.serve_batch_slots, max_batch=args.serve_max_batch)
    out["one_at_a_time"] = serve(1)
    burst = {"requests": args.serve_burst,
             "continuous": serve(args.serve_slots, burst=args.serve_burst),
             "batched": serve(args.serve_batch_slots, max_batch=args.serve_max_batch, burst=args.serve_burst),
             "one_at_a_time": serve(1, burst=args.serve_burst)}
    burst["batched_over_one_at_a_time"] = burst["batched"]["value"] / burst["one_at_a_time"]["value"]
    burst["continuous_over_one_at_a_time"] = burst["continuous"]["value"] / burst["one_at_a_time"]["value"]
    head = out[policies[0]]
    return {"workload": f"Poisson arrivals {args.rate}/s for {args.duration} s ({n} requests); pool of "
                        f"{args.serve_pool} requests of the heterogeneous distribution + 2% large (64x2048^2, "
                        "level 10); inputs in pinned host memory, copied in by the server inside the latency",
            "slots": args.serve_slots, "budget_bytes": 60e9, "requests": n,
            "value": head["value"], "unit": "hulls/s", "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"],
            "policies": out, "served_over_one_at_a_time": head["value"] / out["one_at_a_time"]["value"],
            "p50_one_at_a_time_over_served": out["one_at_a_time"]["p50_ms"] / head["p50_ms"],
            "burst": burst,
            "note": "at 200 requests/s every server keeps up (hulls/s = arrival rate); the burst (all requests "
                    "submitted at once, inputs from pinned host memory) measures each server's capacity"}


def run_serve(args, th, scenes, dev, world, rank):
    m = serve_measure(args, th, scenes, dev, world, rank)
    if rank != 0:
        return None
    return {
        "metric": "hulls/s and p50/p99 ms under Poisson arrivals (continuous batching)", "value": m["value"],
        "unit": "hulls/s", "n_gpus": world, "steps": m["requests"], "warmup": 1, "ms_per_step": 1000.0 / m["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: pregenerated pool of seeded requests replayed by the arrival stream",
        "config": {"workload": m["workload"], "slots": m["slots"], "budget_bytes": m["budget_bytes"]},
        "p50_ms": m["p50_ms"], "p99_ms": m["p99_ms"], "policies": m["policies"], "burst": m["burst"],
        "served_over_one_at_a_time": m["served_over_one_at_a_time"],
    }


def time_calls(fn, n: int, warmup: int) -> tuple[float, list[float]]:
    """(calls/s, sorted per-call ms) of fn on the current stream, CUDA events around each call."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    per: list[float] = []
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        per.append(e0.elapsed_time(e1))
    stop.record()
    torch.cuda.synchronize()
    return n / (start.elapsed_time(stop) / 1000.0), sorted(per)


def reference_cuda_module():
    """torchhull's own CUDA extension (its unmodified sources compiled by oracle/ref_build.py), or None."""
    from oracle import ref_build

    if not ref_build.staged():
        return None
    return ref_build.build()


def reference_cuda_leg(ref, reqs, rounds: int, warmup: int) -> dict:
    """The reference's own CUDA build on the same requests, one per call on the current stream: the
    comparison point for the plain drop-in (its results equal the plain path's bit for bit)."""
    state = {"q": 0}

    def one():
        r = reqs[state["q"] % len(reqs)]
        state["q"] += 1
        ref.visual_hull(*as_tuple(r))

    value, per = time_calls(one, rounds * len(reqs), warmup * len(reqs))
    return {"value": value, "unit": "hulls/s", "p50_ms": percentile(per, 50), "p99_ms": percentile(per, 99),
            "hulls": rounds * len(reqs),
            "path": "torchhull's own CUDA extension built from its unmodified sources (glm/stdgpu stand-ins), "
                    "visual_hull one request per call"}


def headline_extras(args, th, scenes, dev, world, rank, reqs, plain_value) -> dict:
    """The other configurations, measured in the same run (one GPU): the reference CUDA build on the
    headline requests, the small and blur configurations, the 64-request mix and the served stream."""
    import torch

    out: dict = {}
    ref = reference_cuda_module() if not args.no_reference_cuda else None
    if ref is not None:
        leg = reference_cuda_leg(ref, reqs, max(1, min(args.steps, args.ref_rounds)), 1)
        leg["plain_over_reference_cuda"] = plain_value / leg["value"]
        out["reference_cuda"] = leg
    else:
        out["reference_cuda"] = {"unavailable": "reference sources not staged (oracle/_ref/src)"}

    # 8 OpenGL views of 256^2, level 6, full masks
    r1 = scenes.small_request(dev)
    v1, p1 = time_calls(lambda: th.visual_hull(**r1.kwargs()), 50, 5)
    cfg1 = {"workload": "3 ellipsoids, 8 OpenGL views of 256x256 float32, level 6, full masks",
            "plain": {"value": v1, "unit": "hulls/s", "p50_ms": percentile(p1, 50), "p99_ms": percentile(p1, 99)}}
    if ref is not None:
        rv, rp = time_calls(lambda: ref.visual_hull(*as_tuple(r1)), 20, 3)
        cfg1["reference_cuda"] = {"value": rv, "unit": "hulls/s", "p50_ms": percentile(rp, 50)}
        cfg1["plain_over_reference_cuda"] = v1 / rv
    out["cfg1"] = cfg1

    # blur k=9 sigma=2 then level 8, 24 OpenCV views of 512^2
    r2 = scenes.blur_request(device=dev)
    hull_args = (r2.transforms, r2.level, r2.cube_corner_bfl, r2.cube_length, r2.masks_partial,
                 r2.transforms_convention)
    fv, fp = time_calls(lambda: th.visual_hull_blurred(r2.masks, *hull_args, 9, 2.0), 30, 5)
    tv, tp = time_calls(lambda: th.visual_hull(th.gaussian_blur(r2.masks, 9, 2.0), *hull_args), 30, 5)
    cfg2 = {"workload": "5 ellipsoids, 24 OpenCV views of 512x512 float32, gaussian_blur(k=9, sigma=2, sparse), "
                        "visual_hull level 8, full masks",
            "fused": {"value": fv, "unit": "hulls/s", "p50_ms": percentile(fp, 50)},
            "two_calls": {"value": tv, "unit": "hulls/s", "p50_ms": percentile(tp, 50)}}
    if ref is not None:
        rv, rp = time_calls(lambda: ref.visual_hull(ref.gaussian_blur(r2.masks, 9, 2.0, True), *hull_args), 10, 2)
        cfg2["reference_cuda_two_calls"] = {"value": rv, "unit": "hulls/s", "p50_ms": percentile(rp, 50)}
        cfg2["fused_over_reference_cuda"] = fv / rv
    out["cfg2"] = cfg2
    del r1, r2
    torch.cuda.empty_cache()

    if not args.no_hetero:
        out["hetero64"] = hetero_measure(args, th, scenes, dev, world, rank)
        torch.cuda.empty_cache()
    if not args.no_serve:
        out["serve"] = serve_measure(args, th, scenes, dev, world, rank, policies=("none",))
        torch.cuda.empty_cache()
    return out


def octant_args(o: int):
    corner = (-1.0 + (o & 1), -1.0 + (o >> 1 & 1), -1.0 + (o >> 2 & 1))
    return corner, 1.0, LEVEL - 1


def cpu_baseline(req, samples: int = 8) -> dict:
    from oracle import oracle

    masks = req.masks.cpu().numpy()
    tf = req.transforms.cpu().numpy()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for o in range(samples):
        corner, length, level = octant_args(o % 8)
        oracle.visual_hull(masks, tf, level, corner, length, True, "opengl", True, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": (samples / 8.0) / dt, "unit": "hulls/s", "cores": threads, "kind": "port",
            "sample": f"{samples} octants of one request in turn (each level 8 over half the cube: the same "
                      f"leaf size; 8 octants = one hull); {dt:.1f} s"}


def run_reference(args) -> dict | None:
    world, rank, _ = dist_setup()
    if rank != 0:
        return None
    import torch

    from oracle import oracle
    from torchhull_gb300 import scenes

    req = scenes.partial_request(device="cuda" if torch.cuda.is_available() else "cpu", seed=3)
    masks = req.masks.cpu().numpy()
    tf = req.transforms.cpu().numpy()
    threads = os.cpu_count() or 1
    for w in range(args.warmup):
        corner, length, level = octant_args(w % 8)
        oracle.visual_hull(masks, tf, level, corner, length, True, "opengl", True, nthreads=threads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        corner, length, level = octant_args(k % 8)
        oracle.visual_hull(masks, tf, level, corner, length, True, "opengl", True, nthreads=threads)
    total = time.perf_counter() - t0
    value = (args.steps / 8.0) / total
    sample = (f"each step one octant of the cube at the same leaf size (level 8 over half the cube); "
              f"8 steps = one hull; {args.steps} steps in {total:.1f} s")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "hulls/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: seeded ray-ellipsoid/capsule masks",
        "config": {"workload": WORKLOAD,
                   "path": "CPU restatement of the reference algorithm (the reference has no CPU path; its own "
                           "CUDA build is timed as reference_cuda in the GB300 arm's line)"},
        "cpu_baseline": {"value": value, "unit": "hulls/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "hulls/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--mode", choices=["headline", "hetero", "serve", "mc", "blur"], default="headline")
    ap.add_argument("--requests", type=int, default=4)
    ap.add_argument("--cpu-samples", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--carve-kernel", choices=["auto", "views", "items"], default="auto",
                    help="carve kernel: autotuned (default) or forced")
    ap.add_argument("--hetero-count", type=int, default=64)
    ap.add_argument("--hetero-steps", type=int, default=3)
    ap.add_argument("--ref-rounds", type=int, default=5,
                    help="headline: rounds of the Q requests timed through the reference's CUDA build")
    ap.add_argument("--no-extras", action="store_true", help="headline: skip the other configurations")
    ap.add_argument("--no-reference-cuda", action="store_true")
    ap.add_argument("--no-hetero", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--e2e-copy", choices=["dma", "sm"], default="sm",
                    help="plain end-to-end leg: host <-> device copies by the copy kernel or by copy engines")
    ap.add_argument("--e2e-batched-copy", choices=["dma", "sm"], default="dma",
                    help="batched end-to-end leg: copy engines (the copy kernel's few blocks starve beside "
                         "the batch's persistent carve kernel)")
    ap.add_argument("--batch-route", choices=["on", "off"], default="off",
                    help="batched form: requests that fill the GPU alone through the per-request pipeline")
    ap.add_argument("--field-ones", choices=["on", "off"], default="on",
                    help="field without cell masks: test a bitmap of all-ones 2x2 pixel footprints first")
    ap.add_argument("--field-masks", choices=["on", "off"], default="on",
                    help="field: skip the (corner, view) pairs whose factor the carve proved to be 1")
    ap.add_argument("--mc-sizes", default="100,200,300,400,500,600", help="--mode mc: volume sizes")
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--duration", type=float, default=20.0)
    ap.add_argument("--serve-pool", type=int, default=24)
    ap.add_argument("--serve-large", type=int, default=1)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-batch-slots", type=int, default=2, help="batching server: slots (batches in flight)")
    ap.add_argument("--serve-max-batch", type=int, default=16, help="batching server: requests per batch at most")
    ap.add_argument("--serve-burst", type=int, default=384, help="capacity run: requests submitted at once")
    args = ap.parse_args()
    line = run_reference(args) if args.impl == "reference" else run_gb300(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
