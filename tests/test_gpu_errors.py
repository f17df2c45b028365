"""The drop-in's error contract: the reference's checks, raised as RuntimeError with its messages.

Reference: visual_hull_cuda.cu:591-613 (TORCH_CHECK_EQ/GE/GT on dims, sizes,
level and cube length; the convention string), visual_hull.cpp:82 (CPU
tensors), the AT_DISPATCH lists of visual_hull_cuda.cu:646,838-839 (mask and
transform dtypes), gaussian_blur_cuda.cu:294-305 (kernel size, sigma, output
dtype). Where the reference raises through TORCH_CHECK (not a TORCH_CHECK_OP,
which some torch versions turn into a process abort), its own build is called
on the same input and both messages must agree.
"""

from __future__ import annotations

import re

import pytest
import torch

from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def req(cuda):
    return scenes.make_request(40, 4, 64, 4, False, device=cuda)


def call(fn, r, **over):
    a = dict(masks=r.masks, transforms=r.transforms, level=r.level, cube_corner_bfl=r.cube_corner_bfl,
             cube_length=r.cube_length, masks_partial=r.masks_partial,
             transforms_convention=r.transforms_convention, unique_verts=True)
    a.update(over)
    return fn(a["masks"], a["transforms"], a["level"], a["cube_corner_bfl"], a["cube_length"], a["masks_partial"],
              a["transforms_convention"], a["unique_verts"])


CHECK_OP_CASES = {
    # name: (override builder, reference message of visual_hull_cuda.cu:591-599)
    "masks_dims": (lambda r: dict(masks=r.masks[..., 0]), "Check failed: masks.dim() == 4 (3 vs. 4)"),
    "transforms_dims": (lambda r: dict(transforms=r.transforms[0]), "Check failed: transforms.dim() == 3 (2 vs. 3)"),
    "transforms_rows": (lambda r: dict(transforms=r.transforms[:, :3]),
                        "Check failed: transforms.size(1) == 4 (3 vs. 4)"),
    "batch_mismatch": (lambda r: dict(transforms=r.transforms[:3]),
                       "Check failed: masks.size(0) == transforms.size(0) (4 vs. 3)"),
    "channels": (lambda r: dict(masks=r.masks.expand(-1, -1, -1, 2).contiguous()),
                 "Check failed: masks.size(3) == 1 (2 vs. 1)"),
    "level": (lambda r: dict(level=-1), "Check failed: level >= 0 (-1 vs. 0)"),
    "cube_length": (lambda r: dict(cube_length=0.0), "Check failed: cube_length > 0.f (0 vs. 0)"),
}


@pytest.mark.parametrize("name", list(CHECK_OP_CASES))
@pytest.mark.parametrize("entry", ["visual_hull", "visual_hull_with_candidate_voxels", "sparse_visual_hull_field"])
def test_argument_checks(th, req, name, entry):
    over, message = CHECK_OP_CASES[name]
    fn = getattr(th, entry)
    with pytest.raises(RuntimeError, match=re.escape(message)):
        if entry == "sparse_visual_hull_field":
            a = dict(masks=req.masks, transforms=req.transforms, level=req.level, cube_length=req.cube_length)
            a.update(over(req))
            fn(a["masks"], a["transforms"], a["level"], req.cube_corner_bfl, a["cube_length"], False, "opengl")
        else:
            call(fn, req, **over(req))
        torch.cuda.synchronize()


def _messages(fn_ours, fn_ref, *args):
    with pytest.raises(RuntimeError) as ours:
        fn_ours(*args)
    with pytest.raises(RuntimeError) as theirs:
        fn_ref(*args)
    return str(ours.value), str(theirs.value)


def _first_line(msg: str) -> str:
    return msg.strip().splitlines()[0].strip()


def test_unknown_convention_matches_reference(th, ref, req):
    a = (req.masks, req.transforms, 4, req.cube_corner_bfl, 2.0, False, "vulkan", True)
    ours, theirs = _messages(th.visual_hull, ref.visual_hull, *a)
    assert 'Unsupported transforms_convention "vulkan".' in ours
    assert _first_line(ours) == _first_line(theirs)


@pytest.mark.parametrize("entry", ["visual_hull", "visual_hull_with_candidate_voxels", "sparse_visual_hull_field"])
def test_cpu_tensors_match_reference(th, ref, req, entry):
    args = (req.masks.cpu(), req.transforms.cpu(), 4, req.cube_corner_bfl, 2.0, False, "opengl")
    if entry != "sparse_visual_hull_field":
        args = args + (True,)
    ours, theirs = _messages(getattr(th, entry), getattr(ref, entry), *args)
    assert 'No backend implementation available for device "cpu".' in ours
    assert _first_line(ours) == _first_line(theirs)


@pytest.mark.parametrize("dtype", [torch.bool, torch.bfloat16])
def test_unsupported_mask_dtypes_match_reference(th, ref, req, dtype):
    a = (req.masks.to(dtype), req.transforms, 4, req.cube_corner_bfl, 2.0, False, "opengl", True)
    ours, theirs = _messages(th.visual_hull, ref.visual_hull, *a)
    name = {torch.bool: "Bool", torch.bfloat16: "BFloat16"}[dtype]
    assert f"not implemented for '{name}'" in ours
    assert _first_line(ours) == _first_line(theirs)


@pytest.mark.parametrize("dtype", [torch.int32, torch.int64, torch.bfloat16])
def test_unsupported_transform_dtypes_match_reference(th, ref, req, dtype):
    a = (req.masks, req.transforms.to(dtype), 4, req.cube_corner_bfl, 2.0, False, "opengl", True)
    ours, theirs = _messages(th.visual_hull, ref.visual_hull, *a)
    assert "not implemented for" in ours
    assert _first_line(ours) == _first_line(theirs)


@pytest.mark.parametrize("k, sigma, dtype, message", [
    (4, 1.0, None, "kernel_size % 2 == 1"),
    (0, 1.0, None, "kernel_size > 0"),
    (3, 0.0, None, "sigma > 0"),
    (3, 1.0, torch.int32, "isFloatingType"),
])
def test_blur_argument_checks(th, req, k, sigma, dtype, message):
    with pytest.raises(RuntimeError, match=re.escape(message)):
        th.gaussian_blur(req.masks, k, sigma, True, dtype)
