"""The serving scheduler's admission logic on the CPU (no GPU, no contexts).

A server object is assembled without its device parts, and _admit() is
called as a free slot would call it, with the lock held.
"""

from __future__ import annotations

import collections
import concurrent.futures
import threading

import torch

from torchhull_gb300 import serve


def fake_server(budget: int, large: int, max_batch: int, priority: str = "none") -> serve.HullServer:
    s = serve.HullServer.__new__(serve.HullServer)
    s.budget, s.large_bytes, s.max_batch, s.priority = budget, large, max_batch, priority
    s._cv = threading.Condition()
    s._pending = collections.deque()
    s._in_flight = 0
    s._running_bytes = 0
    s._large_running = False
    s._closed = False
    return s


def job(nbytes: int, shape=(2, 8, 8, 1)) -> serve._Job:
    req = serve.HullRequest(torch.zeros(shape), torch.zeros((shape[0], 4, 4)), 3, (-1.0, -1.0, -1.0), 2.0, False,
                            "opengl")
    return serve._Job(req, concurrent.futures.Future(), 0.0, nbytes, None, None)


def test_batches_skip_large_and_over_budget_jobs():
    s = fake_server(budget=100, large=50, max_batch=4)
    big = job(80, (3, 16, 16, 1))           # large: runs alone, stays pending here
    small = [job(10, (2, 8 + i, 8, 1)) for i in range(6)]  # tensors of different shapes
    s._pending.extend([small[0], big] + small[1:])
    with s._cv:
        first = s._admit()
    assert first == [small[0], small[1], small[2], small[3]]
    assert list(s._pending) == [big, small[4], small[5]]
    with s._cv:
        s._in_flight, s._running_bytes = 4, 40
        second = s._admit()  # the large job does not fit beside the running 40 bytes
    assert second == [small[4], small[5]]
    assert list(s._pending) == [big]
    with s._cv:
        s._in_flight, s._running_bytes = 0, 0
        third = s._admit()
    assert third == [big]
    assert not s._pending


def test_one_at_a_time_without_batching():
    s = fake_server(budget=100, large=50, max_batch=1)
    jobs = [job(10) for _ in range(3)]
    s._pending.extend(jobs)
    with s._cv:
        assert s._admit() == [jobs[0]]
        assert s._admit() == [jobs[1]]


def test_jobs_compare_by_identity():
    a, b = job(10), job(10)
    assert a != b and a == a
