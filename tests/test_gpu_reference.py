"""Differential parity against torchhull's own CUDA build, on the same GPU and the same inputs.

``ref`` is the reference's extension compiled from its unmodified sources
(``oracle/ref_build.py``). Every comparison here is exact: per-level candidate
lists in the reference's order, the sparse field's indices and values, the
mesh's vertices and faces, the wireframes. The blur is compared within 1e-5
absolute (the reference's dense blur goes through cuDNN's conv2d, whose
summation order is its own). Where a test also runs the CPU oracle, the oracle
is held to the same exactness, which pins it to the reference's outputs.

Configurations: the 8-view 256^2 level-6 OpenGL scene; the blur + hull scene
(24 views of 512^2, blur k=9 sigma=2, level 8, OpenCV); the partial-view scene
(32 views of 1024^2 at radius 1.4, level 9, partial masks); and smaller
variants for modes, conventions, dtypes and low levels.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle
from torchhull_gb300 import scenes

pytestmark = pytest.mark.gpu

BLUR_TOL = {torch.float16: 1e-3, torch.float32: 1e-5, torch.float64: 1e-5}


def _args(r, masks=None, transforms=None, unique=None):
    return (r.masks if masks is None else masks, r.transforms if transforms is None else transforms, r.level,
            r.cube_corner_bfl, r.cube_length, r.masks_partial, r.transforms_convention,
            r.unique_verts if unique is None else unique)


def _np(t):
    return t.detach().cpu().numpy()


def assert_hull_equal(got, want, what=""):
    """got / want: (verts, faces, candidates) as numpy arrays."""
    gv, gf, gc = got
    wv, wf, wc = want
    assert len(gc) == len(wc), f"{what}: {len(gc)} levels vs {len(wc)}"
    for i, (a, b) in enumerate(zip(gc, wc, strict=True)):
        if not np.array_equal(a, b):
            same_set = a.size == b.size and np.array_equal(np.sort(a), np.sort(b))
            raise AssertionError(f"{what}: level {i} candidates differ ({a.size} vs {b.size}; same set: {same_set})")
    assert gv.shape == wv.shape and gf.shape == wf.shape, f"{what}: mesh {gv.shape}/{gf.shape} vs {wv.shape}/{wf.shape}"
    assert np.array_equal(gf, wf), f"{what}: faces differ"
    assert np.array_equal(gv.view(np.uint32), wv.view(np.uint32)), f"{what}: vertices differ"


def ref_hull(ref, r, **kw):
    v, f, c = ref.visual_hull_with_candidate_voxels(*_args(r, **kw))
    torch.cuda.synchronize()
    return _np(v), _np(f), [_np(x) for x in c]


def our_hull(th, r, **kw):
    v, f, c = th.visual_hull_with_candidate_voxels(*_args(r, **kw))
    torch.cuda.synchronize()
    return _np(v), _np(f), [_np(x) for x in c]


def oracle_hull(r, masks=None, transforms=None, unique=None):
    m = r.masks if masks is None else masks
    t = r.transforms if transforms is None else transforms
    res = oracle.visual_hull(m.cpu(), t.cpu(), r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                             r.transforms_convention, r.unique_verts if unique is None else unique)
    return res.verts, res.faces, res.levels


SCENES = {
    "gl_full_256_l6": lambda dev: scenes.small_request(dev),
    "gl_partial_192_l6": lambda dev: scenes.make_request(21, 12, 192, 6, True, device=dev),
    "cv_full_160_l6": lambda dev: scenes.make_request(22, 10, 160, 6, False, convention="opencv", n_ellipsoids=5,
                                                      device=dev),
    "cv_partial_256_l7": lambda dev: scenes.make_request(26, 16, 256, 7, True, convention="opencv", device=dev),
    "gl_partial_1024_l9": lambda dev: scenes.partial_request(dev),
    # more than 32 views: views 32.. are evaluated without inherited view masks
    "gl_partial_320_l7_40v": lambda dev: scenes.make_request(27, 40, 320, 7, True, device=dev),
    "cv_full_256_l7_48v": lambda dev: scenes.make_request(28, 48, 256, 7, False, convention="opencv", device=dev),
}


@pytest.fixture(scope="module")
def scene_cache(cuda):
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = SCENES[name](cuda)
        return cache[name]

    return get


@pytest.fixture(scope="module")
def blur_scene(cuda, ref):
    """24 OpenCV views of 512^2 blurred by the reference (k=9, sigma=2), hulled at level 8."""
    r = scenes.blur_request(cuda)
    blurred = ref.gaussian_blur(r.masks, 9, 2.0, True)
    torch.cuda.synchronize()
    return r, blurred


@pytest.mark.parametrize("unique", [True, False])
@pytest.mark.parametrize("name", list(SCENES))
def test_hull_matches_reference(th, ref, scene_cache, name, unique):
    r = scene_cache(name)
    want = ref_hull(ref, r, unique=unique)
    assert want[1].shape[0] > 0
    assert_hull_equal(our_hull(th, r, unique=unique), want, name)


@pytest.mark.parametrize("name", ["gl_full_256_l6", "gl_partial_192_l6", "cv_full_160_l6", "cv_partial_256_l7",
                                  "gl_partial_1024_l9", "gl_partial_320_l7_40v"])
def test_oracle_matches_reference(ref, scene_cache, name):
    r = scene_cache(name)
    assert_hull_equal(oracle_hull(r), ref_hull(ref, r), f"oracle {name}")


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name", ["gl_partial_1024_l9", "gl_full_256_l6", "cv_partial_256_l7", "gl_partial_320_l7_40v",
                                  "cv_full_256_l7_48v"])
def test_forced_carve_kernels_match_reference(th, ref, scene_cache, name, mode):
    """Both carve kernels (views over lanes; (parent, view) items with inherited skip masks), each forced."""
    r = scene_cache(name)
    want = ref_hull(ref, r)
    try:
        th._C.set_carve_kernel(0, mode)
        for _ in range(2):
            assert_hull_equal(our_hull(th, r), want, f"{name} carve mode {mode}")
    finally:
        th._C.set_carve_kernel(0, 0)


def test_batched_partial_workload_matches_reference(th, ref, cuda):
    """Four seeded requests of the 32 x 1024^2 level-9 partial workload through the persistent batched carve."""
    reqs = [scenes.partial_request(cuda, seed=3 + i) for i in range(4)]
    got = th._C.visual_hull_batch([_args(r) for r in reqs])
    torch.cuda.synchronize()
    for i, (r, (v, f)) in enumerate(zip(reqs, got, strict=True)):
        wv, wf = ref.visual_hull(*_args(r))
        torch.cuda.synchronize()
        assert torch.equal(f, wf), i
        assert torch.equal(v.view(torch.int32), wv.view(torch.int32)), i


def test_heterogeneous_batch_matches_reference(th, ref, cuda):
    """A batch of the heterogeneous distribution (views 4..48, sides 256..1024, levels 6..9, partial
    or full) without its 1024^2 level-9 requests, through the persistent batched carve."""
    reqs = [r for r in scenes.batched_requests(count=16, seed=5, device=cuda)
            if not (r.level == 9 and r.masks.shape[1] == 1024)][:12]
    assert any(r.masks.shape[0] > 32 for r in reqs)
    got = th._C.visual_hull_batch([_args(r) for r in reqs])
    torch.cuda.synchronize()
    for i, (r, (v, f)) in enumerate(zip(reqs, got, strict=True)):
        wv, wf = ref.visual_hull(*_args(r))
        torch.cuda.synchronize()
        assert torch.equal(f, wf), i
        assert torch.equal(v.view(torch.int32), wv.view(torch.int32)), i


def test_blur_hull_configuration_matches_reference(th, ref, blur_scene):
    r, ref_blurred = blur_scene
    ours = th.gaussian_blur(r.masks, 9, 2.0, True)
    torch.cuda.synchronize()
    assert (ours.double() - ref_blurred.double()).abs().max().item() <= 1e-5
    want = ref_hull(ref, r, masks=ref_blurred)
    assert want[1].shape[0] > 0
    # the hull of the same (reference-blurred) masks
    assert_hull_equal(our_hull(th, r, masks=ref_blurred), want, "blur + hull")
    # the whole chain: this library's blur, then its hull
    assert_hull_equal(our_hull(th, r, masks=ours), want, "blur + hull, own blur")
    # the fused request
    v, f = th.visual_hull_blurred(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length, r.masks_partial,
                                  r.transforms_convention, 9, 2.0, True)
    torch.cuda.synchronize()
    assert np.array_equal(_np(f), want[1]) and np.array_equal(_np(v).view(np.uint32), want[0].view(np.uint32))


def test_blur_hull_oracle_matches_reference(ref, blur_scene):
    r, ref_blurred = blur_scene
    assert np.abs(oracle.gaussian_blur(r.masks.cpu(), 9, 2.0, True) - _np(ref_blurred)).max() <= 1e-5
    assert_hull_equal(oracle_hull(r, masks=ref_blurred), ref_hull(ref, r, masks=ref_blurred), "oracle blur + hull")


@pytest.mark.parametrize("name", ["gl_full_256_l6", "gl_partial_192_l6", "cv_partial_256_l7", "gl_partial_320_l7_40v"])
def test_field_matches_reference(th, ref, scene_cache, name):
    r = scene_cache(name)
    args = _args(r)[:7]
    want = ref.sparse_visual_hull_field(*args).coalesce()
    got = th.sparse_visual_hull_field(*args)
    assert got.shape == want.shape
    assert torch.equal(got.indices(), want.indices())
    assert torch.equal(got.values().view(torch.int32), want.values().view(torch.int32))
    # the oracle's field, as ravelled ids
    res = oracle.visual_hull(r.masks.cpu(), r.transforms.cpu(), *args[2:])
    rr = (1 << r.level) + 1
    idx = _np(want.indices())
    assert np.array_equal(idx[3] + idx[2] * rr + idx[1] * rr * rr, res.field_indices)
    assert np.array_equal(_np(want.values()).view(np.uint32), res.field_values.view(np.uint32))


@pytest.mark.parametrize(
    "mask_dtype", [torch.uint8, torch.int8, torch.int16, torch.int32, torch.int64, torch.float16, torch.float64])
@pytest.mark.parametrize("tf_dtype", [torch.float16, torch.float32, torch.float64])
def test_dtypes_match_reference(th, ref, cuda, mask_dtype, tf_dtype):
    r = scenes.make_request(24, 6, 128, 5, False, device=cuda)
    m = r.masks.to(mask_dtype)
    t = r.transforms.double().to(tf_dtype)
    assert_hull_equal(our_hull(th, r, masks=m, transforms=t), ref_hull(ref, r, masks=m, transforms=t),
                      f"{mask_dtype}/{tf_dtype}")


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("partial", [False, True])
def test_low_levels_match_reference(th, ref, cuda, level, partial):
    r = scenes.make_request(23, 5, 96, level, partial, device=cuda)
    assert_hull_equal(our_hull(th, r), ref_hull(ref, r), f"level {level}")


@pytest.mark.parametrize("partial", [False, True])
@pytest.mark.parametrize("fill", [0.0, 1.0])
def test_constant_masks_match_reference(th, ref, cuda, partial, fill):
    r = scenes.make_request(25, 6, 128, 5, partial, device=cuda)
    m = torch.full_like(r.masks, fill)
    assert_hull_equal(our_hull(th, r, masks=m), ref_hull(ref, r, masks=m), f"fill {fill}")


@pytest.mark.parametrize("kernel_size", [1, 3, 5, 9, 11])
@pytest.mark.parametrize("sparse", [True, False])
@pytest.mark.parametrize("out_dtype", [torch.float16, torch.float32, torch.float64])
def test_blur_matches_reference(th, ref, cuda, kernel_size, sparse, out_dtype):
    m = scenes.make_request(31, 4, 160, 5, False, n_ellipsoids=4, device=cuda).masks
    got = th.gaussian_blur(m, kernel_size, 2.0, sparse, out_dtype)
    want = ref.gaussian_blur(m, kernel_size, 2.0, sparse, out_dtype)
    torch.cuda.synchronize()
    assert got.dtype == want.dtype == out_dtype and got.shape == want.shape
    assert (got.double() - want.double()).abs().max().item() <= BLUR_TOL[out_dtype]


@pytest.mark.parametrize("in_dtype", [torch.uint8, torch.int32, torch.float16, torch.float64])
def test_blur_input_dtypes_match_reference(th, ref, cuda, in_dtype):
    m = scenes.make_request(31, 4, 160, 5, False, n_ellipsoids=4, device=cuda).masks.to(in_dtype)
    got = th.gaussian_blur(m, 9, 2.0, True, torch.float32)
    want = ref.gaussian_blur(m, 9, 2.0, True, torch.float32)
    torch.cuda.synchronize()
    assert (got - want).abs().max().item() <= 1e-5


def _sphere(size, dtype):
    ax = np.linspace(-1.0, 1.0, size)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    return (np.sqrt(x * x + y * y + z * z) - 0.6).astype(dtype)[None]


@pytest.mark.parametrize("sparse", [False, True])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("unique", [True, False])
@pytest.mark.parametrize("local", [True, False])
def test_marching_cubes_matches_reference(th, ref, cuda, sparse, dtype, unique, local):
    sdf = _sphere(33, dtype)
    vol = torch.from_numpy(sdf).to(cuda)
    if sparse:
        keep = np.abs(sdf) < 0.3
        idx = np.stack(np.nonzero(keep)).astype(np.int64)
        vol = torch.sparse_coo_tensor(torch.from_numpy(idx), torch.from_numpy(sdf[keep]), sdf.shape).coalesce()
        vol = vol.to(cuda)
    gv, gf = th.marching_cubes(vol, 0.0, local, unique)
    wv, wf = ref.marching_cubes(vol, 0.0, local, unique)
    torch.cuda.synchronize()
    assert gf.shape == wf.shape and gf.shape[0] > 0
    assert torch.equal(gf, wf)
    assert torch.equal(gv.view(torch.int32), wv.view(torch.int32))


def test_wireframes_match_reference(th, ref, scene_cache):
    r = scene_cache("gl_full_256_l6")
    _, _, cands = ref.visual_hull_with_candidate_voxels(*_args(r))
    want = ref.candidate_voxels_to_wireframes(cands, r.cube_corner_bfl, r.cube_length)
    got = th.candidate_voxels_to_wireframes(cands, r.cube_corner_bfl, r.cube_length)
    torch.cuda.synchronize()
    assert len(got) == len(want)
    for (gv, ge), (wv, we) in zip(got, want, strict=True):
        assert torch.equal(ge, we)
        assert torch.equal(gv.view(torch.int32), wv.view(torch.int32))
