"""The allocation-free blur entry point (th_gaussian_blur_noalloc) through the C ABI.

Callers that cannot call cudaMalloc (a process whose device memory another
framework has reserved, a per-frame loop that must not risk a device-wide
synchronisation, a caller with a fixed device-memory budget) use this variant;
it must give the same images as th_gaussian_blur.  This file is collected
last so that a failure here leaves every other test already run; it passes
alone in a fresh process and after the rest of the suite.
"""

from __future__ import annotations

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the blur tolerance used throughout the tests


@pytest.fixture(scope="module")
def lib():
    from torchhull_gb300 import build

    L = ctypes.CDLL(str(build.LIB))
    L.th_gaussian_blur_noalloc.restype = ctypes.c_int
    L.th_gaussian_blur_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int64, ctypes.c_int32, ctypes.c_float, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    return L


def noalloc_blur(lib, images: torch.Tensor, k: int, sigma: float, sparse: bool, out_dtype: torch.dtype):
    codes = {torch.uint8: 1, torch.int8: 2, torch.int16: 3, torch.int32: 4, torch.int64: 5, torch.float16: 6,
             torch.float32: 7, torch.float64: 8}
    out = torch.empty(images.shape, dtype=out_dtype, device=images.device)
    B, H, W, _ = images.shape
    rc = lib.th_gaussian_blur_noalloc(images.data_ptr(), codes[images.dtype], B, H, W, k, sigma, int(sparse),
                                      out.data_ptr(), codes[out_dtype],
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out


@pytest.mark.parametrize("k", [1, 3, 9])
@pytest.mark.parametrize("out_dtype", [torch.float16, torch.float32, torch.float64])
@pytest.mark.parametrize("sparse", [True, False])
def test_noalloc_matches_blur_twice(cuda, th, lib, sparse, out_dtype, k):
    from torchhull_gb300 import scenes

    first = scenes.make_request(41, views=3, side=200, level=4, partial=False).masks.to(cuda)
    second = scenes.make_request(42, views=5, side=160, level=4, partial=False, n_ellipsoids=5).masks.to(cuda)
    for masks in (first, second):  # two calls in a row: the shared scratch must not leak between calls
        rc, got = noalloc_blur(lib, masks, k, 2.0, sparse, out_dtype)
        torch.cuda.synchronize()
        assert rc == 0
        want = th.gaussian_blur(masks, k, 2.0, sparse, out_dtype)
        assert got.dtype == want.dtype == out_dtype
        assert (got.double() - want.double()).abs().max().item() <= TOL


def test_noalloc_just_below_the_scratch_limit(cuda, th, lib):
    # k=3: B*(H+1)*(W+1) bytes of tile flags + 96 bytes of weights; 4095^2 + 96 = 16,769,121 <= 16 MiB,
    # so the weights sit in the last few kilobytes of the array
    n = 4094
    yy, xx = torch.meshgrid(torch.arange(n, device=cuda), torch.arange(n, device=cuda), indexing="ij")
    disk = (((yy - n / 2) ** 2 + (xx - n / 2) ** 2) < (0.3 * n) ** 2).to(torch.uint8)[None, :, :, None]
    for masks in (disk, 1 - disk):
        rc, got = noalloc_blur(lib, masks.contiguous(), 3, 1.0, True, torch.float32)
        torch.cuda.synchronize()
        assert rc == 0
        want = th.gaussian_blur(masks.contiguous(), 3, 1.0, True, torch.float32)
        assert (got - want).abs().max().item() <= TOL


def test_noalloc_rejects_oversize(cuda, lib):
    # 16 MiB of scratch: one 4096x4096 image with k=3 needs 4097*4097 bytes of tile flags (> 16 MiB)
    big = torch.zeros((1, 4096, 4096, 1), dtype=torch.uint8, device=cuda)
    rc, _ = noalloc_blur(lib, big, 3, 1.0, True, torch.float16)
    assert rc == 1  # TH_ERR_INVALID_ARGUMENT
