"""The CPU oracle against golden outputs of torchhull's own CUDA build.

The fixtures ``tests/golden/ref_*.npz`` were written by
``tests/golden/make_ref_golden.py``, which runs the reference's extension
(compiled from its unmodified sources by ``oracle/ref_build.py``) on a GB300.
They carry their inputs, so these checks need neither a GPU nor the reference
tree: hulls must match bit for bit (per-level candidates in the reference's
order, field, vertices, faces), the blur within 1e-5 absolute, marching cubes
bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests.golden import make_ref_golden as g


def _fixture(name):
    path = g.HERE / f"{name}.npz"
    if not path.exists():
        pytest.fail(f"missing golden fixture {path.name}")
    return g.load(name)


@pytest.mark.parametrize("name", list(g.HULL_CASES))
def test_oracle_hull_matches_reference_golden(name):
    d = _fixture(name)
    level, partial, opengl, unique = (int(x) for x in d["params"])
    res = oracle.visual_hull(g.unpack_masks(d), d["transforms"], level, tuple(float(c) for c in d["corner"]),
                             float(d["length"][0]), bool(partial), "opengl" if opengl else "opencv", bool(unique))
    assert [lv.size for lv in res.levels] == d["level_sizes"].tolist()
    got = {
        "verts": res.verts,
        "faces": res.faces,
        "levels": np.concatenate(res.levels),
        "field_indices": res.field_indices,
        "field_values": res.field_values,
    }
    assert [got["verts"].shape[0], got["faces"].shape[0], got["field_indices"].size] == d["sizes"].tolist()
    for k, a in got.items():
        if k in d:
            assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(d[k]).view(np.uint8)), k
        assert g.digest(a) == str(d[f"sha_{k}"]), k


def test_oracle_blur_matches_reference_golden():
    d = _fixture("ref_blur_96")
    masks = g.unpack_masks(d)
    for k in (3, 9):
        for sparse in (True, False):
            want = d[f"{'sparse' if sparse else 'dense'}_k{k}"]
            got = oracle.gaussian_blur(masks, k, 2.0, sparse, dtype="float32")
            assert np.abs(got - want).max() <= 1e-5, (k, sparse)


def test_oracle_marching_cubes_matches_reference_golden():
    d = _fixture("ref_mc_sphere")
    sdf = g.sphere(int(d["size"][0]))
    keep = np.abs(sdf) < 0.3
    idx = np.stack(np.nonzero(keep)).astype(np.int64)
    for unique in (True, False):
        dense = oracle.marching_cubes(sdf, 0.0, True, unique)
        sparse = oracle.marching_cubes(None, 0.0, True, unique, indices=idx, values=sdf[keep], size=sdf.shape)
        for kind, (v, f) in (("dense", dense), ("sparse", sparse)):
            assert g.digest(v) == str(d[f"{kind}_{int(unique)}_verts"]), (kind, unique)
            assert g.digest(f) == str(d[f"{kind}_{int(unique)}_faces"]), (kind, unique)
