"""Graph replay of the plain pipeline: the same results as direct launches,
for requests of one shape that differ in masks, transforms and cube."""

from __future__ import annotations

import pytest
import torch

from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


def run(th, r, corner=None, length=None):
    kw = r.kwargs()
    if corner is not None:
        kw["cube_corner_bfl"] = corner
        kw["cube_length"] = length
    v, f = th.visual_hull(**kw)
    torch.cuda.synchronize()
    return v.cpu(), f.cpu()


@pytest.mark.parametrize("partial", [False, True])
def test_replays_equal_direct_launches(th, cuda, partial):
    reqs = [scenes.make_request(700 + i, 12, 192, 6, partial, device=cuda) for i in range(3)]
    cubes = [((-1.0, -1.0, -1.0), 2.0), ((-0.9, -1.1, -1.0), 1.9), ((-1.2, -1.0, -0.8), 2.3)]
    try:
        th._C.set_graphs(0, False)
        direct = [run(th, r, *c) for r in reqs for c in cubes]
        th._C.set_graphs(0, True)
        for _ in range(2):  # the first round captures, the second replays
            replay = [run(th, r, *c) for r in reqs for c in cubes]
            for (dv, df), (gv, gf) in zip(direct, replay, strict=True):
                assert torch.equal(dv, gv) and torch.equal(df, gf)
    finally:
        th._C.set_graphs(0, True)


def test_replay_counts_its_kernels(th, cuda):
    r = scenes.make_request(710, 8, 128, 5, False, device=cuda)
    try:
        th._C.set_graphs(0, False)
        run(th, r)
        n0 = th._C.launch_count()
        run(th, r)
        direct = th._C.launch_count() - n0
        th._C.set_graphs(0, True)
        run(th, r)
        n0 = th._C.launch_count()
        run(th, r)
        replay = th._C.launch_count() - n0
    finally:
        th._C.set_graphs(0, True)
    assert direct == replay > 10
