"""GPU parity: the CUDA path against the CPU oracle on the same seeded inputs.

Integer work (occupancy per level, corner set, faces) must match exactly; the
mesh vertices, the hull field and the integral images are computed with the
reference's float operations in the same order, so they are compared for
exact equality too (the stated tolerance, 1e-5 * cube_length for vertices, is
a looser bound than what is checked here).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle
from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu


def run_both(th, cuda, req, unique=True, masks=None, transforms=None):
    masks = req.masks if masks is None else masks
    transforms = req.transforms if transforms is None else transforms
    v, f, cands = th.visual_hull_with_candidate_voxels(
        masks.to(cuda), transforms.to(cuda), req.level, req.cube_corner_bfl, req.cube_length, req.masks_partial,
        req.transforms_convention, unique)
    ref = oracle.visual_hull(masks, transforms, req.level, req.cube_corner_bfl, req.cube_length,
                             req.masks_partial, req.transforms_convention, unique)
    return v.cpu().numpy(), f.cpu().numpy(), [c.cpu().numpy() for c in cands], ref


def assert_same(v, f, cands, ref):
    assert len(cands) == len(ref.levels)
    for i, (a, b) in enumerate(zip(cands, ref.levels, strict=True)):
        assert np.array_equal(a, b), f"level {i} candidates differ ({a.size} vs {b.size})"
    assert v.shape == ref.verts.shape and f.shape == ref.faces.shape
    assert np.array_equal(f, ref.faces)
    assert np.array_equal(v, ref.verts)


@pytest.mark.parametrize("unique", [True, False])
def test_small_config_matches_oracle(th, cuda, unique):
    req = scenes.small_request()
    v, f, cands, ref = run_both(th, cuda, req, unique)
    assert f.shape[0] > 0
    assert_same(v, f, cands, ref)


@pytest.mark.parametrize("unique", [True, False])
def test_partial_matches_oracle(th, cuda, unique):
    req = scenes.make_request(21, views=12, side=192, level=6, partial=True)
    v, f, cands, ref = run_both(th, cuda, req, unique)
    assert f.shape[0] > 0
    assert_same(v, f, cands, ref)


def test_opencv_matches_oracle(th, cuda):
    req = scenes.make_request(22, views=10, side=160, level=6, partial=False, convention="opencv", n_ellipsoids=5)
    v, f, cands, ref = run_both(th, cuda, req)
    assert f.shape[0] > 0
    assert_same(v, f, cands, ref)


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("partial", [False, True])
def test_low_levels(th, cuda, level, partial):
    req = scenes.make_request(23, views=5, side=96, level=level, partial=partial)
    v, f, cands, ref = run_both(th, cuda, req)
    assert_same(v, f, cands, ref)


@pytest.mark.parametrize(
    "mask_dtype", [torch.uint8, torch.int8, torch.int16, torch.int32, torch.int64, torch.float16, torch.float64])
@pytest.mark.parametrize("tf_dtype", [torch.float16, torch.float32, torch.float64])
def test_dtypes(th, cuda, mask_dtype, tf_dtype):
    req = scenes.make_request(24, views=6, side=128, level=5, partial=False)
    v, f, cands, ref = run_both(th, cuda, req, masks=req.masks.to(mask_dtype),
                                transforms=req.transforms.double().to(tf_dtype))
    assert_same(v, f, cands, ref)


@pytest.mark.parametrize("partial", [False, True])
@pytest.mark.parametrize("fill", [0.0, 1.0])
def test_constant_masks_give_empty_mesh(th, cuda, partial, fill):
    # tests/test_visual_hull.py:43-121 of the reference
    req = scenes.make_request(25, views=6, side=128, level=5, partial=partial)
    masks = torch.full_like(req.masks, fill)
    v, f = th.visual_hull(masks.to(cuda), req.transforms.to(cuda), 5, (-1.1, -1.1, -1.1), 2.2, partial, "opengl")
    assert v.shape == (0, 3) and f.shape == (0, 3)
    assert v.dtype == torch.float32 and f.dtype == torch.int64


def test_field_matches_oracle(th, cuda):
    req = scenes.small_request()
    field = th.sparse_visual_hull_field(req.masks.to(cuda), req.transforms.to(cuda), req.level, req.cube_corner_bfl,
                                        req.cube_length, req.masks_partial, req.transforms_convention)
    ref = oracle.visual_hull(req.masks, req.transforms, req.level, req.cube_corner_bfl, req.cube_length,
                             req.masks_partial, req.transforms_convention)
    r = (1 << req.level) + 1
    idx = field.indices().cpu().numpy()
    ravel = idx[3] + idx[2] * r + idx[1] * r * r
    assert field.shape == (1, r, r, r)
    assert np.array_equal(ravel, ref.field_indices)
    assert np.array_equal(field.values().cpu().numpy(), ref.field_values)


@pytest.mark.parametrize("dtype", [torch.uint8, torch.float16, torch.float32, torch.float64])
def test_integral_image_bitwise(th, cuda, dtype):
    g = torch.Generator().manual_seed(5)
    if dtype.is_floating_point:
        masks = torch.rand((3, 97, 131, 1), generator=g).to(dtype)
    else:
        masks = (torch.rand((3, 97, 131, 1), generator=g) > 0.5).to(dtype)
    sat = th.integral_image(masks.to(cuda)).cpu().numpy()
    ref = oracle.integral_image(masks)
    assert np.array_equal(sat.view(np.uint32), ref.view(np.uint32))
    # the reference's own construction, torch.cumsum on the device (visual_hull_cuda.cu:76-90)
    m = masks.to(cuda)
    ref_torch = torch.cumsum(torch.cumsum(m, 1, dtype=torch.float32), 2, dtype=torch.float32)[..., 0].cpu().numpy()
    assert np.array_equal(sat.view(np.uint32), ref_torch.view(np.uint32))


def _cumsum_sat(masks):
    return torch.cumsum(torch.cumsum(masks, 1, dtype=torch.float32), 2, dtype=torch.float32)[..., 0]


@pytest.mark.parametrize("shape", [(32, 1024, 1024), (3, 97, 131), (2, 256, 256), (4, 512, 768), (2, 1000, 1000),
                                   (1, 1024, 2048), (1, 33, 4096), (5, 17, 1)])
@pytest.mark.parametrize("dtype", [torch.uint8, torch.float16, torch.float32, torch.float64])
def test_integral_image_binary_shapes(th, cuda, shape, dtype):
    """0/1 masks take the single pass (banded, look-back carries): equal to torch's cumsum on the device."""
    g = torch.Generator(device=cuda).manual_seed(sum(shape))
    B, H, W = shape
    # a blob plus noise: long runs of ones and zeros, and isolated pixels
    yy, xx = torch.meshgrid(torch.arange(H, device=cuda), torch.arange(W, device=cuda), indexing="ij")
    blob = ((yy - H / 2) ** 2 + (xx - W / 3) ** 2) < (0.3 * max(H, W)) ** 2
    noise = torch.rand((B, H, W), generator=g, device=cuda) < 0.02
    masks = (blob[None] ^ noise).to(dtype)[..., None].contiguous()
    ref = _cumsum_sat(masks)
    assert torch.equal(th.integral_image(masks).view(torch.int32), ref.view(torch.int32))
    # twice: the band scratch (tickets, status words) must come back clean
    assert torch.equal(th.integral_image(masks).view(torch.int32), ref.view(torch.int32))


def test_integral_image_shape_sequence(th, cuda):
    """Calls of different shapes in a row share one scratch whose layout depends on the shape."""
    g = torch.Generator(device=cuda).manual_seed(9)
    for shape in [(16, 1024, 1024), (6, 128, 128), (16, 1024, 1024), (3, 512, 256), (8, 1024, 768)]:
        masks = (torch.rand(shape + (1,), generator=g, device=cuda) < 0.85).float()
        assert torch.equal(th.integral_image(masks).view(torch.int32), _cumsum_sat(masks).view(torch.int32)), shape


@pytest.mark.parametrize("offset", [1, 3])
def test_integral_image_unaligned_masks(th, cuda, offset):
    """Masks starting off a 16-byte boundary are staged without the bulk copy."""
    base = (torch.rand((2 * 256 * 256 + offset,), device=cuda) < 0.5).to(torch.uint8)
    masks = base[offset:].view(2, 256, 256, 1)
    assert torch.equal(th.integral_image(masks).view(torch.int32), _cumsum_sat(masks).view(torch.int32))


def test_integral_image_nonbinary_falls_back(th, cuda):
    """A value other than 0/1 anywhere: the exact sequential passes rebuild the whole table."""
    masks = (torch.rand((4, 512, 512, 1), device=cuda) < 0.5).float()
    masks[2, 300, 17, 0] = 0.25
    assert torch.equal(th.integral_image(masks).view(torch.int32), _cumsum_sat(masks).view(torch.int32))
    binary = (masks > 0.5).float()
    assert torch.equal(th.integral_image(binary).view(torch.int32), _cumsum_sat(binary).view(torch.int32))


@pytest.mark.parametrize("single_pass", [True, False])
def test_sat_option_gives_identical_hulls(th, cuda, single_pass):
    """TH_OPTION_SAT_SINGLE_PASS changes how the integral image is built, not the result."""
    r = scenes.make_request(542, 16, 1024, 8, True, device=cuda)
    want = th.visual_hull(**r.kwargs())
    try:
        th._C.set_sat_single_pass(0, single_pass)
        got = th.visual_hull(**r.kwargs())
    finally:
        th._C.set_sat_single_pass(0, True)
    assert torch.equal(got[1], want[1]) and torch.equal(got[0].view(torch.int32), want[0].view(torch.int32))


def test_arithmetic_probe(cuda):
    """The oracle's float->int64 and fused world-coordinate rules hold on the device."""
    import ctypes

    from tests.probe import build_probe

    lib = ctypes.CDLL(str(build_probe.build()))
    vals = torch.tensor([float("nan"), float("inf"), -float("inf"), 3e38, -3e38, 9.3e18, -9.3e18, 2.5, -2.5, 1e10],
                        dtype=torch.float32, device=cuda)
    out = torch.empty(vals.numel(), dtype=torch.int64, device=cuda)
    v = torch.arange(vals.numel(), dtype=torch.int64, device=cuda) * 37 + 5
    fo = torch.empty(vals.numel(), dtype=torch.float32, device=cuda)
    lib.probe_arithmetic.restype = ctypes.c_int
    lib.probe_arithmetic.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_void_p,
                                        ctypes.c_void_p]
    rc = lib.probe_arithmetic(vals.data_ptr(), out.data_ptr(), vals.numel(), v.data_ptr(), 512.0, -1.1, 2.2,
                                 fo.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rc == 0
    i64 = np.iinfo(np.int64)
    expect = [i64.min, i64.max, i64.min, i64.max, i64.min, i64.max, i64.min, 2, -2, 10000000000]
    assert out.cpu().tolist() == expect
    from fractions import Fraction

    def round_f32(q: Fraction) -> np.float32:
        f = np.float32(float(q))
        cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
        best = min(cands, key=lambda c: (abs(Fraction(float(c)) - q), int(np.float32(c).view(np.uint32)) & 1))
        return np.float32(best)

    L, c = Fraction(float(np.float32(2.2))), Fraction(float(np.float32(-1.1)))
    fused = [round_f32(Fraction(float(np.float32(x) / np.float32(512.0))) * L + c) for x in v.cpu().tolist()]
    assert fo.cpu().numpy().tolist() == [float(x) for x in fused]
