"""Marching cubes on the CPU: the triangulation table's edge property and the
oracle against the reference's own marching-cubes tests
(tests/test_marching_cubes.py: empty input, sphere SDF within 1e-2, closed
2-manifold), dense and sparse, float32 and float64."""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle

TABLE = Path(__file__).resolve().parents[1] / "torchhull_gb300" / "csrc" / "mc_tables.h"


def load_table():
    text = TABLE.read_text()
    counts_txt = re.search(r"TH_MC_TRI_COUNT_INIT \{(.*?)\}", text, re.S).group(1)
    counts = [int(x) for x in re.findall(r"\d+", counts_txt)]
    edges_txt = re.search(r"TH_MC_TRI_EDGES_INIT \{(.*)\}", text, re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", edges_txt)
    edges = [[int(x) for x in re.findall(r"\d+", r)] for r in rows]
    return counts, edges


def test_table_uses_exactly_the_sign_changing_edges():
    """The GPU numbers vertices from per-point edge bits: a cell's table
    vertices must lie on exactly the cell edges whose ends differ in the code."""
    counts, edges = load_table()
    assert len(counts) == 256 and len(edges) == 256
    for code in range(256):
        used = {e for e in edges[code][: counts[code]]}
        want = set()
        for lo in range(8):
            for axis in range(3):
                if (lo >> axis) & 1:
                    continue
                hi = lo | (1 << axis)
                if ((code >> lo) ^ (code >> hi)) & 1:
                    want.add(lo | (axis << 3))
        assert used == want, code
        assert counts[code] % 3 == 0


def sdf_sphere_volume(size: int, dtype=np.float32) -> tuple[np.ndarray, np.ndarray, float]:
    g = np.stack(np.meshgrid(*(3 * [np.arange(size)]), indexing="ij"), 0).reshape(3, -1).T.astype(dtype)
    center = np.full(3, size / 2, dtype=dtype)
    radius = 0.8731945 * (size / 2)
    sdf = (np.linalg.norm(g - center, axis=1) - radius).astype(dtype)
    return sdf.reshape(1, size, size, size), center, radius


def to_sparse(sdf: np.ndarray, truncation: float = 2.0):
    s = sdf.copy()
    s[np.abs(s) > truncation] = 0
    nz = np.nonzero(s)
    indices = np.stack(nz).astype(np.int64)  # rows (0, z, y, x), lexicographic = ascending ravel order
    return indices, s[nz], s.shape


def is_closed_manifold(faces: np.ndarray) -> bool:
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    e.sort(axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    return bool(np.all(counts == 2))


@pytest.mark.parametrize("size", [20, 33])
@pytest.mark.parametrize("sparse", [False, True])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_oracle_sphere(size, sparse, dtype):
    sdf, center, radius = sdf_sphere_volume(size, dtype)
    if sparse:
        idx, vals, shape = to_sparse(sdf)
        verts, faces = oracle.marching_cubes(None, 0.0, False, indices=idx, values=vals, size=shape)
    else:
        verts, faces = oracle.marching_cubes(sdf, 0.0, False)
    d = np.linalg.norm(verts.astype(np.float64) - center, axis=1) - radius
    assert np.abs(d).max() < 2e-2
    assert is_closed_manifold(faces)


@pytest.mark.parametrize("sparse", [False, True])
def test_oracle_empty_input(sparse):
    if sparse:
        v, f = oracle.marching_cubes(None, 0.0, False, indices=np.empty((4, 0), np.int64),
                                     values=np.empty(0, np.float32), size=(1, 10, 10, 10))
    else:
        v, f = oracle.marching_cubes(np.full((1, 10, 10, 10), -1.0, np.float32), 0.0, False)
    assert v.shape == (0, 3) and f.shape == (0, 3)


def test_oracle_soup_and_local_coords():
    sdf, _, _ = sdf_sphere_volume(16)
    vu, fu = oracle.marching_cubes(sdf, 0.0, True, True)
    vs, fs = oracle.marching_cubes(sdf, 0.0, True, False)
    assert fs.shape == fu.shape and vs.shape[0] == 3 * fs.shape[0]
    assert np.array_equal(fs.reshape(-1), np.arange(vs.shape[0]))
    # the soup's corners are the shared vertices, face by face
    assert np.array_equal(vs, vu[fu.reshape(-1)])
    assert vu.min() >= -1.0 and vu.max() <= 1.0
