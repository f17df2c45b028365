"""Wireframes of the candidate voxels and the OBJ/PLY curve-network writer
(torchhull candidate_voxels_to_wireframes, store_curve_network)."""

from __future__ import annotations

import struct

import numpy as np
import pytest
import torch

from oracle import oracle


def expected_obj(verts: np.ndarray, edges: np.ndarray) -> str:
    # io.cpp:28-41: "v x y z" with the default stream format of a float (%g), 1-based "l a b"
    lines = ["v %g %g %g" % tuple(float(x) for x in v) for v in verts]
    lines += ["l %d %d" % (1 + a, 1 + b) for a, b in edges]
    return "".join(line + "\n" for line in lines)


def expected_ply(verts: np.ndarray, edges: np.ndarray) -> bytes:
    head = ("ply\nformat binary_little_endian 1.0\n"
            f"element vertex {len(verts)}\nproperty float x\nproperty float y\nproperty float z\n"
            f"element edge {len(edges)}\nproperty int vertex1\nproperty int vertex2\nend_header\n").encode()
    body = verts.astype("<f4").tobytes() + edges.astype(np.int64).astype("<i4").tobytes()
    return head + body


@pytest.fixture(scope="module")
def network():
    rng = np.random.default_rng(5)
    verts = (rng.normal(size=(37, 3)) * np.array([1e-3, 1.0, 1e4])).astype(np.float32)
    verts[0] = [0.1, -0.0, 1e-8]
    edges = rng.integers(0, 37, size=(50, 2)).astype(np.int64)
    return verts, edges


def test_store_obj_and_ply(th, tmp_path, network):
    verts, edges = network
    net = (torch.from_numpy(verts), torch.from_numpy(edges))
    th.store_curve_network(str(tmp_path / "net.obj"), net)
    assert (tmp_path / "net.obj").read_text() == expected_obj(verts, edges)
    th.store_curve_network(str(tmp_path / "net.ply"), net, verbose=True)
    assert (tmp_path / "net.ply").read_bytes() == expected_ply(verts, edges)
    # the PLY body reads back
    data = (tmp_path / "net.ply").read_bytes()
    body = data[data.index(b"end_header\n") + len(b"end_header\n"):]
    v = np.frombuffer(body[: 12 * len(verts)], dtype="<f4").reshape(-1, 3)
    assert np.array_equal(v, verts)
    assert struct.unpack("<ii", body[12 * len(verts): 12 * len(verts) + 8]) == tuple(int(x) for x in edges[0])


def test_store_unknown_extension(th, tmp_path, network):
    verts, edges = network
    with pytest.raises(RuntimeError, match='No implementation for file extension ".txt"'):
        th.store_curve_network(str(tmp_path / "net.txt"), (torch.from_numpy(verts), torch.from_numpy(edges)))
    with pytest.raises(RuntimeError, match='No implementation for file extension ""'):
        th.store_curve_network(str(tmp_path / "net"), (torch.from_numpy(verts), torch.from_numpy(edges)))


def test_oracle_wireframe_shapes():
    cands = [np.array([0], np.int64), np.array([0, 7], np.int64), np.array([5, 63], np.int64)]
    w = oracle.candidate_voxels_to_wireframes(cands, (-1.0, -1.0, -1.0), 2.0)
    assert [v.shape for v, _ in w] == [(8, 3), (16, 3), (16, 3)]
    v, e = w[1]
    # voxel 7 at level 1 is (1,1,1): its corners span [0, 1]^3
    assert np.array_equal(v[8:].min(axis=0), [0, 0, 0]) and np.array_equal(v[8:].max(axis=0), [1, 1, 1])
    assert e.shape == (24, 2) and e.min() == 0 and e.max() == 15


@pytest.mark.gpu
def test_wireframes_match_oracle(th, cuda):
    from torchhull_gb300 import scenes

    r = scenes.make_request(77, 6, 96, 5, False, device=cuda)
    _, _, cands = th.visual_hull_with_candidate_voxels(**r.kwargs())
    got = th.candidate_voxels_to_wireframes(cands, r.cube_corner_bfl, r.cube_length)
    want = oracle.candidate_voxels_to_wireframes([c.cpu().numpy() for c in cands], r.cube_corner_bfl, r.cube_length)
    assert len(got) == len(want)
    for (gv, ge), (ov, oe) in zip(got, want, strict=True):
        assert gv.dtype == torch.float32 and ge.dtype == torch.int64
        assert np.array_equal(gv.cpu().numpy().view(np.uint32), ov.view(np.uint32))
        assert np.array_equal(ge.cpu().numpy(), oe)


@pytest.mark.gpu
def test_wireframe_errors(th, cuda):
    with pytest.raises(RuntimeError):
        th.candidate_voxels_to_wireframes([], (0.0, 0.0, 0.0), 1.0)
    with pytest.raises(RuntimeError, match="No backend implementation"):
        th.candidate_voxels_to_wireframes([torch.zeros(1, dtype=torch.int64)], (0.0, 0.0, 0.0), 1.0)
    empty = th.candidate_voxels_to_wireframes([torch.zeros(0, dtype=torch.int64, device=cuda)], (0.0, 0.0, 0.0), 1.0)
    assert empty[0][0].shape == (0, 3) and empty[0][1].shape == (0, 2)
