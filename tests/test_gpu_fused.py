"""Fused blur -> hull request: equal, bit for bit, to visual_hull(gaussian_blur(masks, k, sigma), ...)."""

from __future__ import annotations

import pytest
import torch

from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


def two_calls(th, r, k, sigma):
    blurred = th.gaussian_blur(r.masks, k, sigma)
    v, f = th.visual_hull(blurred, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                          r.transforms_convention, r.unique_verts)
    torch.cuda.synchronize()
    return v.cpu(), f.cpu()


def fused(th, r, k, sigma):
    v, f = th.visual_hull_blurred(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                                  r.transforms_convention, k, sigma, r.unique_verts)
    torch.cuda.synchronize()
    return v.cpu(), f.cpu()


def test_blur_configuration(th, cuda):
    # 5 ellipsoids, 24 views of 512^2, level 8, OpenCV, blur k=9 sigma=2
    r = scenes.blur_request(device=cuda)
    ev, ef = two_calls(th, r, 9, 2.0)
    gv, gf = fused(th, r, 9, 2.0)
    assert ef.shape[0] > 0
    assert torch.equal(gv, ev) and torch.equal(gf, ef)


@pytest.mark.parametrize("dtype", [torch.float16, torch.float32, torch.float64])
@pytest.mark.parametrize("partial", [False, True])
def test_small_requests(th, cuda, dtype, partial):
    r = scenes.make_request(610, 8, 128, 6, partial, convention="opengl", device=cuda, mask_dtype=dtype)
    for k, sigma in ((5, 1.0), (9, 2.0)):
        ev, ef = two_calls(th, r, k, sigma)
        gv, gf = fused(th, r, k, sigma)
        assert torch.equal(gv, ev) and torch.equal(gf, ef), (k, sigma)


def test_errors(th, cuda):
    r = scenes.make_request(611, 4, 64, 4, False, device=cuda)
    with pytest.raises(RuntimeError, match="kernel_size % 2 == 1"):
        fused(th, r, 4, 1.0)
    with pytest.raises(RuntimeError, match="sigma > 0"):
        fused(th, r, 5, 0.0)
    ri = scenes.make_request(612, 4, 64, 4, False, device=cuda, mask_dtype=torch.uint8)
    with pytest.raises(RuntimeError, match="isFloatingType"):
        fused(th, ri, 5, 1.0)
