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


@pytest.mark.parametrize("sparse", [True, False])
def test_noalloc_matches_blur_twice(cuda, th, lib, sparse):
    from torchhull_gb300 import scenes

    first = scenes.make_request(41, views=3, side=200, level=4, partial=False).masks.to(cuda)
    second = scenes.make_request(42, views=5, side=160, level=4, partial=False, n_ellipsoids=5).masks.to(cuda)
    for masks in (first, second):  # two calls in a row: the shared scratch must not leak between calls
        rc, got = noalloc_blur(lib, masks, 9, 2.0, sparse, torch.float32)
        torch.cuda.synchronize()
        assert rc == 0
        want = th.gaussian_blur(masks, 9, 2.0, sparse, torch.float32)
        assert (got - want).abs().max().item() <= TOL


def test_noalloc_rejects_oversize(cuda, lib):
    # 16 MiB of scratch: one 4096x4096 image with k=3 needs 4097*4097 bytes of tile flags (> 16 MiB)
    big = torch.zeros((1, 4096, 4096, 1), dtype=torch.uint8, device=cuda)
    rc, _ = noalloc_blur(lib, big, 3, 1.0, True, torch.float16)
    assert rc == 1  # TH_ERR_INVALID_ARGUMENT
