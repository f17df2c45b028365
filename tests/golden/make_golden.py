"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no golden vectors and cannot be built here, so these
fixtures pin the oracle (and, through the GPU tests, the CUDA path) to fixed
outputs on fixed seeded inputs; the oracle itself is checked against the
reference's property tests in tests/test_oracle_cpu.py.

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from torchhull_gb300 import scenes  # noqa: E402

HERE = Path(__file__).resolve().parent

CASES = {
    "hull_gl_full_l5": dict(seed=101, views=8, side=128, level=5, partial=False, convention="opengl"),
    "hull_cv_partial_l5": dict(seed=102, views=10, side=128, level=5, partial=True, convention="opencv"),
    "hull_gl_soup_l4": dict(seed=103, views=6, side=96, level=4, partial=False, convention="opengl", unique=False),
}


def make_hull(name: str, seed: int, views: int, side: int, level: int, partial: bool, convention: str,
              unique: bool = True) -> None:
    req = scenes.make_request(seed, views, side, level, partial, convention)
    masks = req.masks.numpy()
    res = oracle.visual_hull(masks, req.transforms.numpy(), level, req.cube_corner_bfl, req.cube_length, partial,
                             convention, unique)
    np.savez_compressed(
        HERE / f"{name}.npz",
        masks_bits=np.packbits(masks.astype(bool).reshape(-1)),
        masks_shape=np.array(masks.shape),
        transforms=req.transforms.numpy(),
        params=np.array([level, int(partial), int(convention == "opengl"), int(unique)]),
        corner=np.array(req.cube_corner_bfl, dtype=np.float32),
        length=np.array([req.cube_length], dtype=np.float32),
        level_sizes=np.array([lv.size for lv in res.levels]),
        field_indices=res.field_indices,
        field_values=res.field_values,
        verts=res.verts,
        faces=res.faces,
    )


def make_blur() -> None:
    req = scenes.make_request(104, 3, 96, 4, False)
    masks = req.masks.numpy()
    out = {}
    for k in (3, 9):
        out[f"sparse_k{k}"] = oracle.gaussian_blur(masks, k, 2.0, True, dtype="float32")
    np.savez_compressed(HERE / "blur_k3_k9.npz", masks_bits=np.packbits(masks.astype(bool).reshape(-1)),
                        masks_shape=np.array(masks.shape), **out)


def load_hull(name: str) -> dict:
    z = np.load(HERE / f"{name}.npz")
    d = {k: z[k] for k in z.files}
    shape = tuple(d["masks_shape"])
    d["masks"] = np.unpackbits(d["masks_bits"])[: int(np.prod(shape))].reshape(shape).astype(np.float32)
    return d


if __name__ == "__main__":
    for name, kw in CASES.items():
        make_hull(name, **kw)
    make_blur()
    print("fixtures written to", HERE)
