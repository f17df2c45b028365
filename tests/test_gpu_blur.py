"""GPU parity of gaussian_blur against the oracle and the reference's own blur properties.

Tolerance: 1e-5 absolute against the oracle (the oracle calls the host's expf,
the device its own expf; both are within a couple of ulp of exp).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle
from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = {torch.float16: 3e-3, torch.float32: 1e-5, torch.float64: 1e-5}


@pytest.fixture(scope="module")
def masks():
    req = scenes.make_request(31, views=4, side=160, level=5, partial=False, n_ellipsoids=4)
    return req.masks


@pytest.mark.parametrize("kernel_size", [3, 5, 7, 9, 11])
@pytest.mark.parametrize("sparse", [True, False])
@pytest.mark.parametrize("out_dtype", [torch.float16, torch.float32, torch.float64])
def test_blur_matches_oracle(th, cuda, masks, kernel_size, sparse, out_dtype):
    got = th.gaussian_blur(masks.to(cuda), kernel_size, 2.0, sparse, out_dtype).cpu()
    ref = oracle.gaussian_blur(masks, kernel_size, 2.0, sparse, dtype=out_dtype.__repr__().split(".")[1])
    assert got.dtype == out_dtype
    diff = np.abs(got.double().numpy() - ref.astype(np.float64)).max()
    assert diff <= TOL[out_dtype], diff


@pytest.mark.parametrize("in_dtype", [torch.uint8, torch.int8, torch.int16, torch.int32, torch.int64, torch.float16,
                                      torch.float64])
def test_blur_input_dtypes(th, cuda, masks, in_dtype):
    m = masks.to(in_dtype)
    got = th.gaussian_blur(m.to(cuda), 9, 2.0, True, torch.float32).cpu().numpy()
    ref = oracle.gaussian_blur(m, 9, 2.0, True, dtype="float32")
    assert np.abs(got - ref).max() <= 1e-5


@pytest.mark.parametrize("kernel_size", [3, 5, 9, 11])
@pytest.mark.parametrize("sigma", [1.0, 100.0])
@pytest.mark.parametrize("out_dtype", [torch.float16, torch.float32, torch.float64])
def test_dense_equals_sparse(th, cuda, masks, kernel_size, sigma, out_dtype):
    # tests/test_gaussian_blur.py:194-243 of the reference
    m = masks[:, 20:-20, 30:-30, :].contiguous().to(cuda)
    dense = th.gaussian_blur(m, kernel_size, sigma, False, out_dtype)
    sparse = th.gaussian_blur(m, kernel_size, sigma, True, out_dtype)
    eps = {torch.float16: 3e-3, torch.float32: 1e-7, torch.float64: 1e-7}[out_dtype]
    assert torch.allclose(dense, sparse, atol=eps)
    assert torch.all(sparse >= -1e-5) and torch.all(sparse <= 1 + 1e-5)


@pytest.mark.parametrize("sparse", [True, False])
@pytest.mark.parametrize("fill", [0.0, 1.0])
def test_constant_and_identity(th, cuda, masks, sparse, fill):
    m = torch.full_like(masks, fill).to(cuda)
    out = th.gaussian_blur(m, 5, 1.0, sparse, torch.float32)
    assert torch.allclose(out, m.float())
    same = th.gaussian_blur(masks.to(cuda), 1, 1.0, sparse, torch.float64)
    assert torch.equal(same.cpu(), masks.double())


def test_blur_errors(th, cuda, masks):
    m = masks.to(cuda)
    with pytest.raises(RuntimeError):
        th.gaussian_blur(m, 4, 1.0)
    with pytest.raises(RuntimeError):
        th.gaussian_blur(m, 0, 1.0)
    with pytest.raises(RuntimeError):
        th.gaussian_blur(m, 3, 0.0)
    with pytest.raises(RuntimeError):
        th.gaussian_blur(m, 3, 1.0, True, torch.int32)


def test_blur_then_hull(th, cuda):
    """The blur + hull configuration: the hull of the GPU-blurred masks equals the oracle's hull of the same masks."""
    req = scenes.make_request(32, views=8, side=192, level=6, partial=False, convention="opencv", n_ellipsoids=5)
    blurred = th.gaussian_blur(req.masks.to(cuda), 9, 2.0, True)
    ref_blur = oracle.gaussian_blur(req.masks, 9, 2.0, True)
    assert np.abs(blurred.cpu().numpy() - ref_blur).max() <= 1e-5
    v, f = th.visual_hull(blurred, req.transforms.to(cuda), req.level, req.cube_corner_bfl, req.cube_length, False,
                          "opencv", True)
    ref = oracle.visual_hull(blurred.cpu(), req.transforms, req.level, req.cube_corner_bfl, req.cube_length, False,
                             "opencv", True)
    assert np.array_equal(f.cpu().numpy(), ref.faces)
    assert np.array_equal(v.cpu().numpy(), ref.verts)
