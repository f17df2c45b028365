"""Serving form: a continuous-batching request loop for visual hulls on one GPU.

Requests are submitted at any time and return futures. Their masks and
transforms may be on the device (the server's streams wait for the work the
submitting thread had queued on its current stream when it called submit())
or in host memory (copied in on the slot's stream, inside the measured
latency; pinned memory makes the copy asynchronous). Host inputs must stay
unchanged until the request's future resolves.

The server runs up to ``slots`` requests at once, each slot with its own
resident context (SAT, octree and corner pools that stay allocated between
requests) and its own CUDA stream, so the kernels of concurrent requests
overlap on the device.  A request is admitted when a slot
is free and the device memory it needs fits in the admission budget together
with the requests already running; otherwise it waits, and later requests
that do fit may go first (no head-of-line blocking).  With ``max_batch > 1`` a
free slot takes all the pending requests that fit (up to that many) and runs
them as one batch: one persistent carve launch over all their octrees, their
integral images and mesh stages side by side on the slot's context.  Every
request's result is identical to running it alone: the kernels are
deterministic and slots share no state.

The reference has no serving layer; this sits on top of the same C ABI as the
drop-in ``visual_hull``.
"""

from __future__ import annotations

import collections
import concurrent.futures
import dataclasses
import threading
import time

import torch

from . import _C
from .scenes import HullRequest


def _max_nodes(level: int) -> int:
    return sum(8**i for i in range(min(level, 12) + 1))


def estimate_bytes(req: HullRequest) -> int:
    """Device bytes a request holds while it runs: its inputs plus the pools it needs.

    Mirrors the pool sizing of the C library (csrc/capi.cu: prepare): SAT,
    node and corner pools (capped at 16 M entries, the initial capacity), the
    field's all-ones footprint bitmap and cell-mask table, and the corner
    bitmap with its rank words.
    """
    B, H, W = req.masks.shape[:3]
    inputs = req.masks.numel() * req.masks.element_size() + req.transforms.numel() * req.transforms.element_size()
    L = req.level
    R = (1 << L) + 1
    WR = (R + 63) // 64
    nodes = min(_max_nodes(L), 1 << 24)
    corners = min(R**3, 1 << 24)
    parents = min(_max_nodes(L), 1 << 22)
    sat = 4 * B * H * W
    ones = 4 * B * H * ((W + 31) // 32)
    cell_masks = 4 * 8 ** (L - 1) if 1 <= L <= 10 else 0
    node_pool = nodes * (8 + 4 + 4 + 1) + parents * 64
    corner_pool = corners * (8 + 4 + 1 + 1 + 4 + 4)
    bitmap = R * R * WR * (8 + 4) + R * R * 4 + (R * R + 31) // 32 * 4
    return int(inputs + sat + ones + cell_masks + node_pool + corner_pool + bitmap)


@dataclasses.dataclass(eq=False)  # jobs compare by identity (their requests hold tensors)
class _Job:
    req: HullRequest
    future: concurrent.futures.Future
    arrival: float
    bytes: int
    ready: torch.cuda.Event | None  # recorded on the submitter's stream (device inputs)
    consumer: torch.cuda.Stream  # the submitter's current stream, where the results will be used
    started: float = 0.0


class HullServer:
    """Continuous-batching visual-hull server on one device."""

    def __init__(self, device: int = 0, slots: int = 4, budget_bytes: float = 60e9, priority: str = "none",
                 large_bytes: float = 2e9, max_batch: int = 1):
        """priority: how requests above large_bytes of estimated device memory (the ones that set
        the tail latency) share the GPU.  "exclusive_large": a large request waits until the
        running ones finish and then runs alone, and nothing is admitted while it waits or runs;
        "large_first" / "small_first": large / small requests run on high-priority CUDA streams,
        so the block scheduler prefers their kernels; "none": all requests alike.

        max_batch > 1: a slot that becomes free takes up to max_batch of the pending requests that
        fit the budget together and runs them as one batch (th_visual_hull_batch: one persistent
        carve launch over all of their octrees, their integral images and mesh stages side by
        side); requests above large_bytes still run alone.  Results are the same either way."""
        if priority not in ("exclusive_large", "large_first", "small_first", "none"):
            raise ValueError(f"unknown priority policy {priority!r}")
        if max_batch < 1:
            raise ValueError("max_batch must be at least 1")
        self.max_batch = int(max_batch)
        self.device = torch.device("cuda", device)
        self.budget = int(budget_bytes)
        self.priority = priority
        self.large_bytes = int(large_bytes)
        self._cv = threading.Condition()
        self._pending: collections.deque[_Job] = collections.deque()
        self._in_flight = 0
        self._running_bytes = 0
        self._large_running = False
        self._closed = False
        self.latencies_ms: list[float] = []
        self.queue_ms: list[float] = []
        self.completed = 0
        self._contexts = [_C.HullContext(device) for _ in range(slots)]
        self._streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self._streams_hi = [torch.cuda.Stream(self.device, priority=-1) for _ in range(slots)]
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(slots)]
        for t in self._threads:
            t.start()

    # -- client side ---------------------------------------------------------
    def submit(self, req: HullRequest) -> concurrent.futures.Future:
        """Queues a request; the future resolves to (verts, faces) on the device.

        The results are complete when the future resolves and may be used on
        the stream that was current in the submitting thread (the server
        records that use with the caching allocator); other streams must
        synchronise with it first."""
        need = estimate_bytes(req)
        if need > self.budget:
            raise ValueError(f"request needs {need} bytes, more than the admission budget {self.budget}")
        fut: concurrent.futures.Future = concurrent.futures.Future()
        consumer = torch.cuda.current_stream(self.device)
        ready = None
        if req.masks.is_cuda or req.transforms.is_cuda:
            ready = torch.cuda.Event()
            ready.record(consumer)
        with self._cv:
            if self._closed:
                raise RuntimeError("server is closed")
            self._pending.append(_Job(req, fut, time.perf_counter(), need, ready, consumer))
            self._cv.notify_all()
        return fut

    def warm_up(self, requests: list[HullRequest]) -> None:
        """Runs every request once on every slot's context (and, with batching, in batches of
        max_batch), synchronously: each context then has its pools sized, its carve kernel tuned
        and its CUDA graphs captured for these request shapes before timed traffic arrives.
        Call it before submitting requests."""
        for slot, ctx in enumerate(self._contexts):
            stream = self._streams[slot]
            with torch.cuda.stream(stream):
                args = [(r.masks.to(self.device, non_blocking=True), r.transforms.to(self.device, non_blocking=True),
                         r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial, r.transforms_convention,
                         r.unique_verts) for r in requests]
                for a in args:
                    ctx.visual_hull(*a)
                if self.max_batch > 1:
                    small = [a for a, r in zip(args, requests, strict=True) if estimate_bytes(r) <= self.large_bytes]
                    for i in range(0, len(small), self.max_batch):
                        ctx.visual_hull_batch(small[i:i + self.max_batch])
            stream.synchronize()

    def close(self) -> None:
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self) -> HullServer:
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def stats(self) -> dict:
        lat = sorted(self.latencies_ms)

        def pct(p: float) -> float | None:
            if not lat:
                return None
            return lat[min(len(lat) - 1, int(round(p / 100.0 * (len(lat) - 1))))]

        return {"completed": self.completed, "p50_ms": pct(50), "p99_ms": pct(99),
                "mean_queue_ms": (sum(self.queue_ms) / len(self.queue_ms)) if self.queue_ms else None,
                "pool_bytes": sum(c.device_bytes() for c in self._contexts)}

    # -- server side ---------------------------------------------------------
    def _is_large(self, job: _Job) -> bool:
        return job.bytes > self.large_bytes

    def _admit_one(self) -> _Job | None:
        """First pending job that fits the budget (called with the lock held)."""
        exclusive = self.priority == "exclusive_large"
        if exclusive and self._large_running:
            return None
        for i, job in enumerate(self._pending):
            if exclusive and self._is_large(job):
                if self._in_flight > 0:
                    return None  # drain the running requests, admit nothing meanwhile
                del self._pending[i]
                self._large_running = True
                return job
            if self._running_bytes + job.bytes <= self.budget or self._in_flight == 0:
                del self._pending[i]
                return job
        return None

    def _admit(self) -> list[_Job]:
        """The jobs a free slot runs next (called with the lock held): the first pending job that
        fits, and with batching the further small pending jobs that fit beside it."""
        first = self._admit_one()
        if first is None:
            return []
        jobs = [first]
        if self.max_batch > 1 and not self._is_large(first):
            need = first.bytes
            keep: collections.deque[_Job] = collections.deque()
            while self._pending:
                job = self._pending.popleft()
                if (len(jobs) < self.max_batch and not self._is_large(job)
                        and self._running_bytes + need + job.bytes <= self.budget):
                    jobs.append(job)
                    need += job.bytes
                else:
                    keep.append(job)
            self._pending = keep
        return jobs

    def _stream_for(self, slot: int, job: _Job) -> torch.cuda.Stream:
        large = job.bytes > self.large_bytes
        hi = (self.priority == "large_first" and large) or (self.priority == "small_first" and not large)
        return self._streams_hi[slot] if hi else self._streams[slot]

    def _worker(self, slot: int) -> None:
        ctx = self._contexts[slot]
        while True:
            with self._cv:
                jobs: list[_Job] = []
                try:
                    while not jobs:
                        jobs = self._admit()
                        if not jobs:
                            if self._closed and not self._pending:
                                return
                            self._cv.wait()
                except Exception as exc:  # a broken scheduler must not leave callers waiting
                    for job in list(self._pending) + jobs:
                        if not job.future.done():
                            job.future.set_exception(exc)
                    self._pending.clear()
                    self._closed = True
                    self._cv.notify_all()
                    return
                self._in_flight += len(jobs)
                self._running_bytes += sum(job.bytes for job in jobs)
            started = time.perf_counter()
            for job in jobs:
                job.started = started
            stream = self._stream_for(slot, jobs[0])
            try:
                with torch.cuda.stream(stream):
                    args = []
                    for job in jobs:
                        r = job.req
                        if job.ready is not None:
                            stream.wait_event(job.ready)
                        masks = r.masks.to(self.device, non_blocking=True)
                        transforms = r.transforms.to(self.device, non_blocking=True)
                        args.append((masks, transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                                     r.transforms_convention, r.unique_verts))
                    outs = [ctx.visual_hull(*args[0])] if len(jobs) == 1 else ctx.visual_hull_batch(args)
                    for job, (verts, faces) in zip(jobs, outs, strict=True):
                        if job.consumer != stream:
                            verts.record_stream(job.consumer)
                            faces.record_stream(job.consumer)
                stream.synchronize()
                done = time.perf_counter()
                for job, out in zip(jobs, outs, strict=True):
                    job.future.set_result(tuple(out))
                with self._cv:
                    for job in jobs:
                        self.latencies_ms.append(1000.0 * (done - job.arrival))
                        self.queue_ms.append(1000.0 * (job.started - job.arrival))
                    self.completed += len(jobs)
            except Exception as exc:  # surfaced to the callers through the futures
                for job in jobs:
                    if not job.future.done():
                        job.future.set_exception(exc)
            finally:
                with self._cv:
                    self._in_flight -= len(jobs)
                    self._running_bytes -= sum(job.bytes for job in jobs)
                    if self.priority == "exclusive_large" and any(self._is_large(job) for job in jobs):
                        self._large_running = False
                    self._cv.notify_all()
