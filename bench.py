"""Benchmark of the visual-hull path: hulls/s on the level-9, 32x1024^2 partial-view workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step"): the visual hull of Q requests (default 4), each a
distinct seeded scene of 8 ellipsoids + 20 thin capsules seen by 32 cameras at
radius 1.4 (fov 50 deg, OpenGL convention) as float32 masks [32,1024,1024,1],
masks_partial=True, level 9, unique vertices.  The masks are synthetic (ray
tests at pixel centres) and stand in for the reference's OpenGL-rendered
dataset.  Each request's masks are 128 MiB, so inputs exceed L2 between
timed iterations.

GB300 arm: inputs resident in HBM; every hull goes through the public
drop-in (torchhull_gb300.visual_hull, i.e. the C ABI).  `value` is hulls/s
of the whole job, `e2e` the same metric with the masks copied from pinned
host memory and the mesh copied back inside the timed region.  Stage times
come from CUDA events the library records between stages on the request's
stream; the largest stage is the roofline line.  Under torchrun every rank
serves its own requests (weak scaling, no collective on the data path).

Reference arm: the reference has no CPU path and its CUDA build cannot be
built here, so it times the CPU restatement of the reference's algorithm
(oracle/) with all host threads.  One step is one octant of the cube at the
same leaf size (level 8 over half the cube length): 8 steps cover one hull.
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

LEVEL = 9
VIEWS = 32
SIDE = 1024
METRIC = "hulls/s, level 9, 32x1024^2 views, partial masks (p50/p99 ms per hull alongside)"
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"


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
                      mask_bytes: int) -> dict:
    """Per-stage algorithmic bytes of one hull (the formula of the design notes)."""
    out = {"integral_image": (mask_bytes + 4) * B * H * W}
    carve = []
    for i in range(len(info_levels) - 1):
        p, pn = info_levels[i], info_levels[i + 1]
        carve.append(8 * p + 8 * p * B * 16 + 8 * pn)
    out["carve"] = carve
    leaves = info_levels[-1]
    out["corners"] = 8 * 8 * leaves + 8 * corners
    out["field"] = corners * B * 16 + 4 * corners + 8 * corners
    out["marching_cubes"] = corners * (16 + 8 * 16) + 12 * verts + 24 * faces
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
    Q = args.requests
    reqs = [scenes.partial_request(device=dev, seed=3 + 1000 * rank + q) for q in range(Q)]
    torch.cuda.synchronize()

    def hull(r):
        return th.visual_hull(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                              r.transforms_convention, r.unique_verts)

    for _ in range(args.warmup):
        for r in reqs:
            hull(r)
    torch.cuda.synchronize()

    th._C.set_profiling(local, True)
    stage_acc: dict[str, list] = {}
    per_hull_ms: list[float] = []
    sizes = []
    sampler = ClockSampler(local)
    launches0 = th._C.launch_count()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        for r in reqs:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            v, f = hull(r)
            e1.record()
            e1.synchronize()
            per_hull_ms.append(e0.elapsed_time(e1))
            st = th._C.stage_times(local)
            for k, val in st.items():
                stage_acc.setdefault(k, []).append(val)
            sizes.append((v.shape[0], f.shape[0]))
    stop.record()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    launches = th._C.launch_count() - launches0
    th._C.set_profiling(local, False)
    elapsed_ms = start.elapsed_time(stop)
    t = torch.tensor([elapsed_ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    hulls = Q * args.steps * world
    value = hulls / (max_ms / 1000.0)

    # end to end: masks from pinned host memory in, mesh out, inside the timed region
    host_masks = [r.masks.cpu().pin_memory() for r in reqs]
    host_tf = [r.transforms.cpu().pin_memory() for r in reqs]
    dev_masks = [torch.empty_like(r.masks) for r in reqs]
    dev_tf = [torch.empty_like(r.transforms) for r in reqs]
    h2d = sum(m.numel() * m.element_size() for m in host_masks) + sum(x.numel() * x.element_size() for x in host_tf)
    d2h_total = 0
    e2e_steps = max(1, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for q, r in enumerate(reqs):
            dev_masks[q].copy_(host_masks[q], non_blocking=True)
            dev_tf[q].copy_(host_tf[q], non_blocking=True)
            v, f = th.visual_hull(dev_masks[q], dev_tf[q], r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                                  r.transforms_convention, r.unique_verts)
            vh = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
            fh = torch.empty(f.shape, dtype=f.dtype, pin_memory=True)
            vh.copy_(v, non_blocking=True)
            fh.copy_(f, non_blocking=True)
            d2h_total += vh.numel() * 4 + fh.numel() * 8
        torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    t = torch.tensor([e2e_s], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = Q * e2e_steps * world / float(t.item())

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return None

    # roofline from the stage events of the timed region
    info = th.visual_hull_with_candidate_voxels(reqs[0].masks, reqs[0].transforms, LEVEL, reqs[0].cube_corner_bfl,
                                                reqs[0].cube_length, True, "opengl", True)
    levels = [c.numel() for c in info[2]]
    field = th.sparse_visual_hull_field(reqs[0].masks, reqs[0].transforms, LEVEL, reqs[0].cube_corner_bfl,
                                        reqs[0].cube_length, True, "opengl")
    corners = field.values().numel()
    nv, nf = info[0].shape[0], info[1].shape[0]
    algo = algorithmic_bytes(levels, corners, nv, nf, VIEWS, SIDE, SIDE, 4)
    mean = {k: (statistics.fmean(v) if not isinstance(v[0], list) else [statistics.fmean(x) for x in zip(*v)])
            for k, v in stage_acc.items()}
    candidates = [("integral_image", "sat_columns_kernel+sat_rows_kernel", mean["integral_image"],
                   algo["integral_image"])]
    for i, ms in enumerate(mean["carve"]):
        candidates.append((f"carve_level_{i}", "classify_kernel+scan", ms, algo["carve"][i]))
    candidates += [("corners", "mark_corners_kernel+scans", mean["corners"], algo["corners"]),
                   ("field", "field_kernel", mean["field"], algo["field"]),
                   ("marching_cubes", "mc_cells_kernel+scan", mean["marching_cubes"], algo["marching_cubes"])]
    dom = max(candidates, key=lambda c: c[2])
    peak, peak_kind = peaks()
    achieved = dom[3] / (dom[2] / 1000.0) / 1e9
    per_hull_ms.sort()

    def pct(p):
        return per_hull_ms[min(len(per_hull_ms) - 1, int(round(p / 100.0 * (len(per_hull_ms) - 1))))]

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "hulls/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: seeded ray-ellipsoid/capsule masks (stand-in for the reference's rendered dataset)",
        "config": {"workload": "partial-view visual hull: 32 views of 1024x1024 float32 masks, level 9, "
                               "masks_partial=True, unique_verts=True, OpenGL, 8 ellipsoids + 20 capsules",
                   "requests_per_step": Q, "level": LEVEL, "views": VIEWS, "side": SIDE,
                   "l2": "inputs larger than L2 (128 MiB of masks + 128 MiB SAT per request)",
                   "path": "plain drop-in visual_hull per request (C ABI)",
                   "mesh_verts": nv, "mesh_faces": nf, "leaves": levels[-1], "corners": corners},
        "p50_ms": pct(50),
        "p99_ms": pct(99),
        "stage_ms": mean,
        "e2e": {"value": e2e_value, "unit": "hulls/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h_total // e2e_steps},
        "roofline": {"bound": "hbm", "kernel": dom[1], "stage": dom[0], "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": dom[3], "ms": dom[2], "traffic": None},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(reqs[0], samples=args.cpu_samples)
    if world > 1:
        dist.destroy_process_group()
    return line


def octant_args(o: int):
    corner = (-1.0 + (o & 1), -1.0 + (o >> 1 & 1), -1.0 + (o >> 2 & 1))
    return corner, 1.0, LEVEL - 1


def cpu_baseline(req, samples: int = 2) -> dict:
    from oracle import oracle

    masks = req.masks.cpu().numpy()
    tf = req.transforms.cpu().numpy()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for o in range(samples):
        corner, length, level = octant_args(o)
        oracle.visual_hull(masks, tf, level, corner, length, True, "opengl", True, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": (samples / 8.0) / dt, "unit": "hulls/s", "cores": threads, "kind": "port",
            "sample": f"{samples} of the 8 octants of one request (same leaf size: level 8 over half the cube); "
                      f"{dt:.1f} s"}


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
    times = []
    t0 = time.perf_counter()
    for k in range(args.steps):
        corner, length, level = octant_args(k % 8)
        s = time.perf_counter()
        oracle.visual_hull(masks, tf, level, corner, length, True, "opengl", True, nthreads=threads)
        times.append(time.perf_counter() - s)
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
        "config": {"workload": "partial-view visual hull: 32 views of 1024x1024 float32 masks, level 9, "
                               "masks_partial=True, unique_verts=True, OpenGL, 8 ellipsoids + 20 capsules",
                   "path": "CPU restatement of the reference algorithm (the reference has no CPU path and its "
                           "CUDA build needs glm/stdgpu/charonload, absent offline)"},
        "cpu_baseline": {"value": value, "unit": "hulls/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "hulls/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--requests", type=int, default=4)
    ap.add_argument("--cpu-samples", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--carve-kernel", choices=["auto", "views", "items"], default="auto",
                    help="carve kernel: autotuned (default) or forced")
    args = ap.parse_args()
    line = run_reference(args) if args.impl == "reference" else run_gb300(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
