"""Marching cubes on the GPU against the oracle, bit for bit, plus the
reference's own checks (tests/test_marching_cubes.py)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle

from test_mc_cpu import is_closed_manifold, sdf_sphere_volume, to_sparse

pytestmark = pytest.mark.gpu

TORCH_DTYPES = {np.float16: torch.float16, np.float32: torch.float32, np.float64: torch.float64}


def gpu_mc(th, cuda, sdf, sparse, iso, local, unique, dtype):
    if sparse:
        idx, vals, shape = to_sparse(sdf)
        vol = torch.sparse_coo_tensor(torch.from_numpy(idx), torch.from_numpy(vals).to(TORCH_DTYPES[dtype]),
                                      shape).coalesce().to(cuda)
    else:
        vol = torch.from_numpy(sdf).to(TORCH_DTYPES[dtype]).to(cuda)
    v, f = th.marching_cubes(vol, iso, local, unique)
    torch.cuda.synchronize()
    return v.cpu().numpy(), f.cpu().numpy()


def oracle_mc(sdf, sparse, iso, local, unique, dtype):
    sdf = sdf.astype(dtype)
    if sparse:
        idx, vals, shape = to_sparse(sdf)
        return oracle.marching_cubes(None, iso, local, unique, indices=idx, values=vals, size=shape)
    return oracle.marching_cubes(sdf, iso, local, unique)


@pytest.mark.parametrize("size", [20, 33])
@pytest.mark.parametrize("sparse", [False, True])
@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.float64])
@pytest.mark.parametrize("unique", [True, False])
@pytest.mark.parametrize("local", [False, True])
def test_sphere_matches_oracle(th, cuda, size, sparse, dtype, unique, local):
    sdf, _, _ = sdf_sphere_volume(size, np.float64)
    sdf = sdf.astype(dtype)
    gv, gf = gpu_mc(th, cuda, sdf, sparse, 0.0, local, unique, dtype)
    ov, of = oracle_mc(sdf, sparse, 0.0, local, unique, dtype)
    assert gv.shape == ov.shape and gf.shape == of.shape
    assert np.array_equal(gf, of)
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32))


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("iso", [0.0, 0.3])
@pytest.mark.parametrize("sparse", [False, True])
def test_noise_volume_matches_oracle(th, cuda, seed, iso, sparse):
    # every cell configuration, including the ambiguous ones, and values on the isolevel
    rng = np.random.default_rng(seed)
    sdf = rng.normal(0.3, 0.5, size=(1, 17, 17, 17)).astype(np.float32)
    sdf[rng.random(sdf.shape) < 0.05] = iso
    if sparse:
        sdf[np.abs(sdf) > 0.9] = 0
    for unique in (True, False):
        gv, gf = gpu_mc(th, cuda, sdf, sparse, iso, False, unique, np.float32)
        ov, of = oracle_mc(sdf, sparse, iso, False, unique, np.float32)
        assert np.array_equal(gf, of)
        assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32))


@pytest.mark.parametrize("shape", [(12, 7, 12), (9, 14, 5), (6, 6, 21)])
@pytest.mark.parametrize("sparse", [False, True])
def test_non_cubic_matches_oracle(th, cuda, shape, sparse):
    rng = np.random.default_rng(3)
    sdf = rng.normal(0.0, 1.0, size=(1, *shape)).astype(np.float32)
    if sparse:
        sdf[np.abs(sdf) > 1.2] = 0
    gv, gf = gpu_mc(th, cuda, sdf, sparse, 0.1, True, True, np.float32)
    ov, of = oracle_mc(sdf, sparse, 0.1, True, True, np.float32)
    assert np.array_equal(gf, of)
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32))


@pytest.mark.parametrize("size", [100, 200])
@pytest.mark.parametrize("sparse", [False, True])
def test_reference_sphere_check(th, cuda, size, sparse):
    # tests/test_marching_cubes.py:67-99 at its first sizes
    sdf, center, radius = sdf_sphere_volume(size, np.float32)
    gv, gf = gpu_mc(th, cuda, sdf, sparse, 0.0, False, True, np.float32)
    d = np.linalg.norm(gv.astype(np.float64) - center, axis=1) - radius
    assert np.abs(d).max() < 1e-2
    assert is_closed_manifold(gf)


@pytest.mark.parametrize("sparse", [False, True])
def test_empty_input(th, cuda, sparse):
    if sparse:
        vol = torch.sparse_coo_tensor(torch.empty([4, 0], dtype=torch.int64), torch.empty([0]),
                                      [1, 100, 100, 100]).to(cuda)
    else:
        vol = torch.full([1, 100, 100, 100], -1.0, device=cuda)
    v, f = th.marching_cubes(vol, isolevel=0, return_local_coords=False)
    assert v.shape == (0, 3) and f.shape == (0, 3)
    assert v.dtype == torch.float32 and f.dtype == torch.int64


def test_errors(th, cuda):
    vol = torch.zeros([1, 8, 8, 8], device=cuda)
    with pytest.raises(RuntimeError, match="isolevel >= 0"):
        th.marching_cubes(vol, -1.0)
    with pytest.raises(RuntimeError, match="dim"):
        th.marching_cubes(vol[0], 0.0)
    with pytest.raises(RuntimeError, match="not implemented for 'Int'"):
        th.marching_cubes(torch.zeros([1, 8, 8, 8], dtype=torch.int32, device=cuda), 0.0)
    with pytest.raises(RuntimeError, match="No backend implementation"):
        th.marching_cubes(vol.cpu(), 0.0)
    with pytest.raises((RuntimeError, IndexError)):
        th.marching_cubes(torch.zeros([1, 1, 8, 8], device=cuda), 0.0)
    unco = torch.sparse_coo_tensor(torch.tensor([[0, 0], [1, 1], [1, 1], [1, 1]]), torch.tensor([1.0, 2.0]),
                                   [1, 4, 4, 4]).to(cuda)
    with pytest.raises(RuntimeError):
        th.marching_cubes(unco, 0.0)
    # the context stays usable
    v, f = th.marching_cubes(torch.from_numpy(sdf_sphere_volume(16)[0]).to(cuda), 0.0)
    assert f.shape[0] > 0
