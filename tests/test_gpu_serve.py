"""Serving form: results in the mix equal results alone; admission by memory budget."""

from __future__ import annotations

import pytest
import torch

from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def requests(cuda):
    out = []
    for i, (views, side, level, partial) in enumerate(
            [(6, 128, 5, False), (12, 192, 6, True), (4, 96, 4, False), (9, 160, 6, False), (16, 256, 7, True),
             (5, 128, 5, True), (8, 256, 6, False), (20, 128, 6, True)]):
        out.append(scenes.make_request(300 + i, views, side, level, partial, device=cuda))
    return out


def alone(th, r):
    v, f = th.visual_hull(**r.kwargs())
    torch.cuda.synchronize()
    return v.cpu(), f.cpu()


@pytest.mark.parametrize("priority", ["exclusive_large", "large_first", "small_first", "none"])
def test_results_in_the_mix_equal_results_alone(th, cuda, requests, priority):
    from torchhull_gb300.serve import HullServer

    expected = [alone(th, r) for r in requests]
    # large_bytes splits the mix so both stream priorities carry requests
    with HullServer(device=cuda.index or 0, slots=3, budget_bytes=20e9, priority=priority,
                    large_bytes=2e8) as server:
        futures = [server.submit(r) for r in requests + requests]
        got = [f.result(timeout=120) for f in futures]
        stats = server.stats()
    for k, (v, f) in enumerate(got):
        ev, ef = expected[k % len(requests)]
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef), k
    assert stats["completed"] == 2 * len(requests)
    assert stats["p50_ms"] is not None and stats["p99_ms"] >= stats["p50_ms"]


def test_tight_budget_admits_one_at_a_time(th, cuda, requests):
    from torchhull_gb300.serve import HullServer, estimate_bytes

    budget = max(estimate_bytes(r) for r in requests)  # room for one request at a time
    with HullServer(device=cuda.index or 0, slots=3, budget_bytes=budget) as server:
        futures = [server.submit(r) for r in requests[:4]]
        got = [f.result(timeout=120) for f in futures]
    for r, (v, f) in zip(requests[:4], got, strict=True):
        ev, ef = alone(th, r)
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)


def test_request_larger_than_budget_is_refused(cuda, requests):
    from torchhull_gb300.serve import HullServer

    with HullServer(device=cuda.index or 0, slots=1, budget_bytes=1e6) as server:
        with pytest.raises(ValueError):
            server.submit(requests[0])


def test_unknown_priority_policy_is_refused(cuda):
    from torchhull_gb300.serve import HullServer

    with pytest.raises(ValueError):
        HullServer(device=cuda.index or 0, slots=1, priority="fastest")


def test_submit_without_synchronizing(th, cuda, requests):
    """Inputs still being written on the submitting thread's stream are waited for, not read early."""
    from torchhull_gb300.serve import HullServer

    expected = [alone(th, r) for r in requests[:4]]
    side = torch.cuda.Stream(cuda)
    with torch.cuda.stream(side), HullServer(device=cuda.index or 0, slots=2) as server:
        futures = []
        for r in requests[:4]:
            busy = torch.randn(4096, 4096, device=cuda)
            for _ in range(8):  # keep the stream busy before the masks are written
                busy = busy @ busy.T / 4096.0
            masks = torch.zeros_like(r.masks)
            masks.copy_(r.masks)
            futures.append(server.submit(scenes.HullRequest(masks, r.transforms, r.level, r.cube_corner_bfl,
                                                            r.cube_length, r.masks_partial,
                                                            r.transforms_convention)))
            del masks
        got = [f.result(timeout=120) for f in futures]
        got = [(v.cpu(), f.cpu()) for v, f in got]
    for (v, f), (ev, ef) in zip(got, expected, strict=True):
        assert torch.equal(v, ev) and torch.equal(f, ef)


def test_host_inputs_are_copied_in(th, cuda, requests):
    from torchhull_gb300.serve import HullServer

    host = [scenes.HullRequest(r.masks.cpu().pin_memory(), r.transforms.cpu(), r.level, r.cube_corner_bfl,
                               r.cube_length, r.masks_partial, r.transforms_convention) for r in requests]
    with HullServer(device=cuda.index or 0, slots=3) as server:
        got = [f.result(timeout=120) for f in [server.submit(r) for r in host]]
    for r, (v, f) in zip(requests, got, strict=True):
        ev, ef = alone(th, r)
        assert v.is_cuda and torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)


@pytest.mark.parametrize("large_bytes", [2e9, 2e8])
@pytest.mark.parametrize("host", [False, True])
def test_batched_serving_equals_results_alone(th, cuda, requests, host, large_bytes):
    """max_batch > 1: requests pending together run as one batch on a slot's context; with the
    smaller large_bytes some requests count as large, run alone and are skipped by the batches."""
    from torchhull_gb300.serve import HullServer

    reqs = requests + requests
    if host:
        reqs = [scenes.HullRequest(r.masks.cpu().pin_memory(), r.transforms.cpu(), r.level, r.cube_corner_bfl,
                                   r.cube_length, r.masks_partial, r.transforms_convention) for r in reqs]
    expected = [alone(th, r) for r in requests]
    with HullServer(device=cuda.index or 0, slots=2, budget_bytes=20e9, max_batch=8,
                    large_bytes=large_bytes) as server:
        futures = [server.submit(r) for r in reqs]
        got = [f.result(timeout=120) for f in futures]
        stats = server.stats()
    for k, (v, f) in enumerate(got):
        ev, ef = expected[k % len(requests)]
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef), k
    assert stats["completed"] == len(reqs)


def test_batch_on_a_private_context(th, cuda, requests):
    """HullContext.visual_hull_batch equals the plain drop-in on each request."""
    ctx = th._C.HullContext(cuda.index or 0)
    tuples = [(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
               r.transforms_convention, r.unique_verts) for r in requests]
    for _ in range(2):
        got = ctx.visual_hull_batch(tuples)
        for r, (v, f) in zip(requests, got, strict=True):
            ev, ef = alone(th, r)
            assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)


def test_warm_up_then_serve(th, cuda, requests):
    from torchhull_gb300.serve import HullServer

    with HullServer(device=cuda.index or 0, slots=2, max_batch=4) as server:
        server.warm_up(requests[:3])
        got = [f.result(timeout=120) for f in [server.submit(r) for r in requests[:3]]]
    for r, (v, f) in zip(requests[:3], got, strict=True):
        ev, ef = alone(th, r)
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)
