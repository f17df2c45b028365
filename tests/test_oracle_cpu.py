"""CPU checks of the oracle: the reference's own property tests and known answers.

The reference's tests (tests/test_visual_hull.py, tests/test_gaussian_blur.py)
pin properties, not values; they are restated here against the oracle on the
synthetic scenes that stand in for the reference's OpenGL-rendered dataset.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle
from torchhull_gb300 import scenes


def is_closed_manifold(faces: np.ndarray) -> bool:
    # tests/test_visual_hull.py:22-29 of the reference
    edges = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    edges = np.sort(edges, axis=1)
    _, counts = np.unique(edges, axis=0, return_counts=True)
    return bool(np.all(counts == 2))


@pytest.fixture(scope="module")
def small():
    return scenes.make_request(7, views=8, side=128, level=5, partial=False)


@pytest.mark.parametrize("level", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("partial", [False, True])
@pytest.mark.parametrize("dtype", [torch.int8, torch.int16, torch.int32, torch.int64, torch.float16, torch.float32,
                                   torch.float64])
def test_empty_and_full_masks(small, level, partial, dtype):
    # tests/test_visual_hull.py:43-121
    for fill in (0, 1):
        masks = torch.full_like(small.masks, fill).to(dtype)
        res = oracle.visual_hull(masks, small.transforms, level, (-1.1, -1.1, -1.1), 2.2, partial, "opengl")
        assert res.verts.shape == (0, 3) and res.faces.shape == (0, 3)


@pytest.fixture(scope="module")
def framed():
    # Cameras far enough out that the object stays inside every frame, as the
    # reference's dataset does.  (Where an object leaves a frame, full mode
    # clamps the SAT box to the image but samples zeros outside it, which
    # leaves an open seam; that is the reference's behaviour too.)
    return scenes.make_request(7, views=8, side=128, level=5, partial=False, radius=4.0)


@pytest.mark.parametrize("level", [1, 3, 5, 6])
@pytest.mark.parametrize("unique", [True, False])
def test_mesh_properties(framed, level, unique):
    # tests/test_visual_hull.py:124-165
    res = oracle.visual_hull(framed.masks, framed.transforms, level, (-1.1, -1.1, -1.1), 2.2, False, "opengl", unique)
    assert level < 3 or res.faces.shape[0] > 0
    assert np.all(res.verts >= -1.1) and np.all(res.verts <= 1.1)
    if unique:
        assert is_closed_manifold(res.faces)
    else:
        assert res.verts.shape[0] == 3 * res.faces.shape[0]
        # soup faces are arange(V) with columns 1 and 2 swapped (visual_hull_cuda.cu:941-956)
        assert np.array_equal(res.faces, np.arange(res.verts.shape[0]).reshape(-1, 3)[:, [0, 2, 1]])


def test_vertices_lie_on_grid_edges(small):
    # marching cubes puts every vertex on a grid edge: two of three grid coordinates are integers
    level = 5
    res = oracle.visual_hull(small.masks, small.transforms, level, (-1.0, -1.0, -1.0), 2.0, False, "opengl")
    g = (res.verts.astype(np.float64) + 1.0) / 2.0 * (1 << level)
    near_int = np.abs(g - np.round(g)) < 1e-4
    assert np.all(near_int.sum(axis=1) >= 2)


@pytest.mark.parametrize("level", [1, 2, 3, 4])
@pytest.mark.parametrize("partial", [False, True])
def test_opengl_and_opencv_agree(level, partial):
    # tests/test_visual_hull.py:168-249: same scene and cameras in both conventions
    seed, views, side = 9, 8, 96
    scene = scenes.make_scene(seed, 3)
    out = {}
    for conv in ("opengl", "opencv"):
        cams = scenes.make_cameras(seed, views, 2.5, 40.0, side, side, conv)
        masks = scenes.render_masks(scene, cams)
        tf = torch.as_tensor(cams.transforms, dtype=torch.float32)
        out[conv] = oracle.visual_hull(masks, tf, level, (-1.1, -1.1, -1.1), 2.2, partial, conv)
    gl, cv = out["opengl"].verts, out["opencv"].verts
    assert level < 3 or gl.shape[0] > 0
    assert (gl.shape[0] == 0) == (cv.shape[0] == 0)
    if gl.shape[0] == 0:
        return
    d = np.linalg.norm(gl[:, None, :] - cv[None, :, :], axis=2).min(axis=1)
    assert np.all(d < 1e-4)


def test_candidates_nest(small):
    # tests/test_visual_hull.py:306-368: every candidate lies inside a candidate of the level above
    res = oracle.visual_hull(small.masks, small.transforms, 5, (-1.0, -1.0, -1.0), 2.0, True, "opengl")
    for i in range(1, len(res.levels)):
        r, rp = 1 << i, 1 << (i - 1)
        c = res.levels[i]
        x, y, z = c % r, c // r % r, c // (r * r)
        parents = (x // 2) + (y // 2) * rp + (z // 2) * rp * rp
        assert np.all(np.isin(parents, res.levels[i - 1]))


def test_integral_image_known_answer():
    rng = np.random.default_rng(3)
    m = (rng.random((2, 37, 53, 1)) > 0.4).astype(np.float32)
    sat = oracle.integral_image(m)
    exact = m[..., 0].astype(np.int64).cumsum(1).cumsum(2)
    assert np.array_equal(sat.astype(np.int64), exact)


def test_integral_image_sequential_float32():
    # torch's CUDA cumsum over a non-innermost dim adds one float32 element at a
    # time (the GPU tests compare against it directly); numpy's accumulate does
    # the same on the host.  (torch's CPU cumsum accumulates in double instead.)
    g = torch.Generator().manual_seed(4)
    m = torch.rand((3, 41, 29, 1), generator=g)
    a = m[..., 0].numpy()
    ref = np.cumsum(np.cumsum(a, axis=1, dtype=np.float32), axis=2, dtype=np.float32)
    sat = oracle.integral_image(m)
    assert np.array_equal(sat.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("sparse", [True, False])
@pytest.mark.parametrize("in_dtype", [torch.int8, torch.int64, torch.float16, torch.float32, torch.float64])
@pytest.mark.parametrize("out_dtype", ["float16", "float32", "float64"])
def test_blur_identity_cases(sparse, in_dtype, out_dtype):
    # tests/test_gaussian_blur.py:22-117: empty, full and k=1 are identities
    rng = np.random.default_rng(1)
    m = torch.from_numpy((rng.random((2, 24, 20, 1)) > 0.5).astype(np.float32)).to(in_dtype)
    for masks, k in ((torch.zeros_like(m), 5), (torch.ones_like(m), 5), (m, 1)):
        out = oracle.gaussian_blur(masks, k, 1.0, sparse, dtype=out_dtype)
        assert out.dtype == np.dtype(out_dtype)
        assert np.allclose(out.astype(np.float64), masks.double().numpy())


@pytest.mark.parametrize("kernel_size", [3, 5, 7, 9, 11])
@pytest.mark.parametrize("sigma", [1.0, 100.0])
def test_blur_dense_equals_sparse_and_range(kernel_size, sigma):
    # tests/test_gaussian_blur.py:118-243
    req = scenes.make_request(13, 2, 64, 4, False)
    dense = oracle.gaussian_blur(req.masks, kernel_size, sigma, False, dtype="float32")
    sparse = oracle.gaussian_blur(req.masks, kernel_size, sigma, True, dtype="float32")
    assert np.allclose(dense, sparse, atol=1e-7)
    assert sparse.min() >= -1e-5 and sparse.max() <= 1 + 1e-5


def test_blur_errors():
    m = np.zeros((1, 8, 8, 1), np.float32)
    for k, s, dt in ((4, 1.0, None), (0, 1.0, None), (3, 0.0, None), (3, 1.0, "int32")):
        with pytest.raises(RuntimeError):
            oracle.gaussian_blur(m, k, s, True, dtype=dt)


def test_hull_argument_errors(small):
    with pytest.raises(RuntimeError):
        oracle.visual_hull(small.masks, small.transforms, -1, (-1, -1, -1), 2.0, False, "opengl")
    with pytest.raises(RuntimeError):
        oracle.visual_hull(small.masks, small.transforms, 3, (-1, -1, -1), 0.0, False, "opengl")
    with pytest.raises(ValueError):
        oracle.visual_hull(small.masks, small.transforms, 3, (-1, -1, -1), 2.0, False, "vulkan")
    with pytest.raises(RuntimeError):
        oracle.visual_hull(small.masks.to(torch.bool), small.transforms, 3, (-1, -1, -1), 2.0, False, "opengl")


def test_thread_count_does_not_change_results(small):
    a = oracle.visual_hull(small.masks, small.transforms, 5, (-1, -1, -1), 2.0, True, "opengl", nthreads=1)
    b = oracle.visual_hull(small.masks, small.transforms, 5, (-1, -1, -1), 2.0, True, "opengl", nthreads=8)
    assert np.array_equal(a.verts, b.verts) and np.array_equal(a.faces, b.faces)


def test_bilerp_of_ones_is_exactly_one():
    """The GPU field returns 1 for a sample whose 2x2 footprint is all ones
    without interpolating; that needs bilerp(1, 1, 1, 1, t, t) == 1 for every
    float32 weight in [0, 1] (checked over [0, 1.25], every value).  Negative
    weights are excluded by the shortcut and do fail."""
    L = oracle.lib()
    one_and_a_quarter = int(np.array(1.25, np.float32).view(np.uint32))
    assert L.oracle_bilerp_ones_failures(0, one_and_a_quarter) == 0
    minus = int(np.array(-(2.0**-25) * (1 + 2.0**-23), np.float32).view(np.uint32))
    assert L.oracle_bilerp_ones_failures(minus, minus + 16) > 0
