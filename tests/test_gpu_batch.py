"""Batched form: every request of a batch equals the plain drop-in on that request, bit for bit."""

from __future__ import annotations

import pytest
import torch

from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


def plain(th, r):
    v, f = th.visual_hull(**r.kwargs())
    torch.cuda.synchronize()
    return v.cpu(), f.cpu()


def as_tuple(r):
    return (r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
            r.transforms_convention, r.unique_verts)


def test_heterogeneous_batch_matches_plain(th, cuda):
    # uneven view counts, sizes, levels, modes and conventions in one batch
    specs = [(4, 96, 4, False, "opengl"), (12, 192, 6, True, "opengl"), (7, 128, 5, False, "opencv"),
             (20, 160, 6, False, "opengl"), (5, 256, 7, True, "opencv"), (33, 96, 5, True, "opengl"),
             (9, 128, 0, False, "opengl"), (6, 64, 1, True, "opengl"), (16, 256, 7, False, "opengl")]
    reqs = [scenes.make_request(500 + i, v, s, lv, part, convention=conv, device=cuda)
            for i, (v, s, lv, part, conv) in enumerate(specs)]
    reqs[2].unique_verts = False
    expected = [plain(th, r) for r in reqs]
    for _ in range(2):  # twice: the resident pools must come back clean
        got = th._C.visual_hull_batch([as_tuple(r) for r in reqs])
        torch.cuda.synchronize()
        for k, ((v, f), (ev, ef)) in enumerate(zip(got, expected, strict=True)):
            assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef), k


def test_batch_with_degenerate_requests(th, cuda):
    base = scenes.make_request(520, 6, 96, 4, False, device=cuda)
    empty = scenes.HullRequest(torch.zeros_like(base.masks), base.transforms, 4, (-1.0, -1.0, -1.0), 2.0, False,
                               "opengl")
    full = scenes.HullRequest(torch.ones_like(base.masks), base.transforms, 5, (-1.0, -1.0, -1.0), 2.0, True,
                              "opengl")
    reqs = [base, empty, full, base]
    got = th._C.visual_hull_batch([as_tuple(r) for r in reqs])
    for r, (v, f) in zip(reqs, got, strict=True):
        ev, ef = plain(th, r)
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)
    assert got[1][1].shape == (0, 3) and got[2][1].shape == (0, 3)


def test_level9_batch_matches_plain(th, cuda):
    reqs = [scenes.make_request(530 + i, 24, 512, 9, i % 2 == 0, device=cuda) for i in range(3)]
    expected = [plain(th, r) for r in reqs]
    got = th._C.visual_hull_batch([as_tuple(r) for r in reqs])
    for (v, f), (ev, ef) in zip(got, expected, strict=True):
        assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)


@pytest.mark.parametrize("route", [True, False])
def test_gpu_filling_requests_routed_or_shared(th, cuda, route):
    # level 8 with 16 views of 1024^2 fills the GPU alone: routed through the
    # per-request pipeline when routing is on, through the shared carve when off
    reqs = [scenes.make_request(540, 16, 1024, 8, False, device=cuda),
            scenes.make_request(541, 6, 128, 5, True, device=cuda),
            scenes.make_request(542, 16, 1024, 8, True, device=cuda)]
    expected = [plain(th, r) for r in reqs]
    try:
        th._C.set_batch_route(0, route)
        for _ in range(2):
            got = th._C.visual_hull_batch([as_tuple(r) for r in reqs])
            for (v, f), (ev, ef) in zip(got, expected, strict=True):
                assert torch.equal(v.cpu(), ev) and torch.equal(f.cpu(), ef)
    finally:
        th._C.set_batch_route(0, False)


def test_batch_and_plain_calls_from_two_threads(th, cuda):
    """A batch on one thread and plain calls on another share the device's context without deadlocking."""
    import threading

    reqs = [scenes.make_request(550 + i, 16, 256, 7, i % 2 == 0, device=cuda) for i in range(4)]
    expected = [plain(th, r) for r in reqs]
    errors: list[BaseException] = []
    results: dict[str, list] = {"batch": [], "plain": []}

    def batches():
        try:
            for _ in range(4):
                out = th._C.visual_hull_batch([as_tuple(r) for r in reqs])
                torch.cuda.synchronize()
                results["batch"].append([(v.cpu(), f.cpu()) for v, f in out])
        except BaseException as exc:  # reported below
            errors.append(exc)

    def plains():
        try:
            for _ in range(4):
                results["plain"].append([plain(th, r) for r in reqs])
        except BaseException as exc:
            errors.append(exc)

    threads = [threading.Thread(target=batches, daemon=True), threading.Thread(target=plains, daemon=True)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in threads), "threads did not finish"
    assert not errors, errors
    for run in results["batch"] + results["plain"]:
        for (v, f), (ev, ef) in zip(run, expected, strict=True):
            assert torch.equal(v, ev) and torch.equal(f, ef)
