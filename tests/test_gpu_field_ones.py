"""The field's two exact shortcuts: the cell masks from the carve
(TH_OPTION_FIELD_MASKS: (corner, view) pairs whose factor is exactly 1 are
skipped) and, where there are none, the all-ones footprint bitmap
(TH_OPTION_FIELD_ONES: a sample whose 2x2 mask footprint is all ones returns
1 without reading the masks).  Field values and meshes must be bit-identical
with and without them: full and partial masks, binary and blurred
(non-binary) masks, every mask dtype, OpenCV, more than 32 views, widths that
are no multiple of 32, NaN projections, the batched form, and the oracle."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle
from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu

CASES = {
    "partial_32": dict(seed=41, views=32, side=256, level=7, partial=True),
    "full_12": dict(seed=42, views=12, side=192, level=6, partial=False),
    "partial_40": dict(seed=43, views=40, side=160, level=6, partial=True),
    "partial_opencv_20": dict(seed=44, views=20, side=192, level=6, partial=True, convention="opencv"),
    "full_opencv_33": dict(seed=45, views=33, side=128, level=6, partial=False, convention="opencv"),
    # widths that are no multiple of 32: the bitmap comes from its own kernel,
    # not from the integral-image pass
    "partial_150": dict(seed=49, views=14, side=150, level=6, partial=True),
    "full_97": dict(seed=50, views=9, side=97, level=6, partial=False),
}


def field_and_mesh(th, cuda, r, masks=None, transforms=None):
    masks = (r.masks if masks is None else masks).to(cuda)
    tf = (r.transforms if transforms is None else transforms).to(cuda)
    field = th.sparse_visual_hull_field(masks, tf, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                                        r.transforms_convention).coalesce()
    v, f = th.visual_hull(masks, tf, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                          r.transforms_convention, True)
    torch.cuda.synchronize()
    return (field.indices().cpu().numpy(), field.values().cpu().numpy().view(np.uint32),
            v.cpu().numpy().view(np.uint32), f.cpu().numpy())


# (cell masks, all-ones bitmap): plain evaluation, the bitmap alone, the default
VARIANTS = [(False, False), (False, True), (True, True)]


def set_variant(th, masks, ones):
    th._C.set_field_masks(0, masks)
    th._C.set_field_ones(0, ones)


def on_off(th, cuda, r, **kw):
    results = []
    try:
        for masks, ones in VARIANTS:
            set_variant(th, masks, ones)
            results.append(field_and_mesh(th, cuda, r, **kw))
    finally:
        set_variant(th, True, True)
    for other in results[1:]:
        for x, y in zip(other, results[0], strict=True):
            assert x.shape == y.shape
            assert np.array_equal(x, y)
    return results[-1]


@pytest.mark.parametrize("case", sorted(CASES))
def test_shortcut_does_not_change_results(th, cuda, case):
    on = on_off(th, cuda, scenes.make_request(**CASES[case]))
    assert on[3].shape[0] > 0


def test_shortcut_matches_oracle(th, cuda):
    r = scenes.make_request(**CASES["partial_32"])
    idx, val, v, f = field_and_mesh(th, cuda, r)
    ref = oracle.visual_hull(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, True, "opengl")
    assert np.array_equal(f, ref.faces)
    assert np.array_equal(v, ref.verts.view(np.uint32))
    assert np.array_equal(val, ref.field_values.view(np.uint32))


@pytest.mark.parametrize("partial", [False, True])
def test_blurred_masks(th, cuda, partial):
    r = scenes.make_request(46, views=16, side=192, level=6, partial=partial)
    on_off(th, cuda, r, masks=th.gaussian_blur(r.masks.to(cuda), 5, 1.5))


@pytest.mark.parametrize("dtype", [torch.uint8, torch.int32, torch.float16, torch.float64])
def test_mask_dtypes(th, cuda, dtype):
    r = scenes.make_request(47, views=24, side=160, level=6, partial=False)
    on_off(th, cuda, r, masks=r.masks.to(dtype))


def test_nan_projections(th, cuda):
    # an all-zero transform projects every point to 0/0 = NaN; in full mode
    # the reference's sample is then NaN, which the shortcut must not replace
    r = scenes.make_request(48, views=6, side=128, level=5, partial=False)
    tf = r.transforms.clone()
    tf[2] = 0
    on_off(th, cuda, r, transforms=tf)


def test_batched(th, cuda):
    reqs = [scenes.make_request(**CASES[c]) for c in sorted(CASES)]
    tuples = [(r.masks.to(cuda), r.transforms.to(cuda), r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
               r.transforms_convention, True) for r in reqs]
    results = []
    try:
        for masks, ones in VARIANTS:
            set_variant(th, masks, ones)
            results.append([(v.cpu().numpy(), f.cpu().numpy()) for v, f in th._C.visual_hull_batch(tuples)])
    finally:
        set_variant(th, True, True)
    for other in results[1:]:
        for (va, fa), (vb, fb) in zip(other, results[0], strict=True):
            assert np.array_equal(fa, fb)
            assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
