"""Writes golden fixtures from torchhull's own CUDA build (run on a machine with a GPU).

The reference extension is compiled from torchhull's unmodified sources by
``oracle/ref_build.py``. This script runs it on fixed, seeded inputs and
stores the inputs with its outputs, so that ``tests/test_ref_golden_cpu.py``
can hold the CPU oracle to the reference's results on any machine:

* small hulls: every per-level candidate list, the sparse field and the mesh
  as full arrays;
* larger hulls (the 8-view 256^2 level-6 scene, a 16-view 512^2 level-8
  partial scene): SHA-256 digests of the same arrays, plus their sizes;
* the blur of a small mask stack (sparse and dense, k = 3 and 9) as arrays;
* marching cubes of a sampled sphere, dense and sparse, as digests.

    python tests/golden/make_ref_golden.py [output directory]
"""

from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
HERE = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# (seed, views, side, level, partial, convention, unique, full arrays?)
HULL_CASES = {
    "ref_gl_full_128_l5": (101, 8, 128, 5, False, "opengl", True, True),
    "ref_cv_partial_128_l5": (102, 10, 128, 5, True, "opencv", True, True),
    "ref_gl_soup_96_l4": (103, 6, 96, 4, False, "opengl", False, True),
    "ref_gl_full_256_l6": (1, 8, 256, 6, False, "opengl", True, False),
    "ref_gl_partial_512_l8": (105, 16, 512, 8, True, "opengl", True, False),
}
BLUR_SEED = 104
SPHERE_SIZE = 33


def digest(a: np.ndarray) -> str:
    """SHA-256 over dtype, shape and the bytes of a C-contiguous array."""
    a = np.ascontiguousarray(a)
    h = hashlib.sha256()
    h.update(a.dtype.str.encode())
    h.update(str(a.shape).encode())
    h.update(a.tobytes())
    return h.hexdigest()


def sphere(size: int, dtype=np.float32) -> np.ndarray:
    ax = np.linspace(-1.0, 1.0, size)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    return (np.sqrt(x * x + y * y + z * z) - 0.6).astype(dtype)[None]


def unpack_masks(d: dict) -> np.ndarray:
    shape = tuple(int(s) for s in d["masks_shape"])
    return np.unpackbits(d["masks_bits"])[: int(np.prod(shape))].reshape(shape).astype(np.float32)


def load(name: str) -> dict:
    z = np.load(HERE / f"{name}.npz")
    return {k: z[k] for k in z.files}


def main(out_dir: Path) -> None:
    import torch

    from oracle import ref_build
    from torchhull_gb300 import scenes

    ref = ref_build.build()
    if ref is None:
        raise SystemExit("reference sources are not staged (oracle/_ref/src)")
    dev = torch.device("cuda:0")
    out_dir.mkdir(parents=True, exist_ok=True)

    for name, (seed, views, side, level, partial, conv, unique, full) in HULL_CASES.items():
        req = scenes.make_request(seed, views, side, level, partial, conv)
        masks = req.masks.numpy()
        args = (req.cube_corner_bfl, req.cube_length, partial, conv)
        v, f, cands = ref.visual_hull_with_candidate_voxels(req.masks.to(dev), req.transforms.to(dev), level, *args,
                                                            unique)
        field = ref.sparse_visual_hull_field(req.masks.to(dev), req.transforms.to(dev), level, *args).coalesce()
        torch.cuda.synchronize()
        r = (1 << level) + 1
        idx = field.indices().cpu().numpy()
        arrays = {
            "verts": v.cpu().numpy(),
            "faces": f.cpu().numpy(),
            "levels": np.concatenate([c.cpu().numpy() for c in cands]),
            "field_indices": idx[3] + idx[2] * r + idx[1] * r * r,
            "field_values": field.values().cpu().numpy(),
        }
        payload = dict(
            masks_bits=np.packbits(masks.astype(bool).reshape(-1)),
            masks_shape=np.array(masks.shape),
            transforms=req.transforms.numpy(),
            params=np.array([level, int(partial), int(conv == "opengl"), int(unique)]),
            corner=np.array(req.cube_corner_bfl, dtype=np.float32),
            length=np.array([req.cube_length], dtype=np.float32),
            level_sizes=np.array([c.numel() for c in cands]),
            sizes=np.array([arrays["verts"].shape[0], arrays["faces"].shape[0], arrays["field_indices"].size]),
        )
        for k, a in arrays.items():
            if full:
                payload[k] = a
            payload[f"sha_{k}"] = np.array(digest(a))
        np.savez_compressed(out_dir / f"{name}.npz", **payload)
        print(name, "faces", arrays["faces"].shape[0], "levels", payload["level_sizes"].tolist())

    req = scenes.make_request(BLUR_SEED, 3, 96, 4, False)
    masks = req.masks.numpy()
    blur = {}
    for k in (3, 9):
        for sparse in (True, False):
            o = ref.gaussian_blur(req.masks.to(dev), k, 2.0, sparse, torch.float32)
            blur[f"{'sparse' if sparse else 'dense'}_k{k}"] = o.cpu().numpy()
    np.savez_compressed(out_dir / "ref_blur_96.npz", masks_bits=np.packbits(masks.astype(bool).reshape(-1)),
                        masks_shape=np.array(masks.shape), **blur)

    sdf = sphere(SPHERE_SIZE)
    mc = {}
    vol = torch.from_numpy(sdf).to(dev)
    keep = np.abs(sdf) < 0.3
    sp_idx = np.stack(np.nonzero(keep)).astype(np.int64)
    svol = torch.sparse_coo_tensor(torch.from_numpy(sp_idx), torch.from_numpy(sdf[keep]), sdf.shape).coalesce()
    for kind, vv in (("dense", vol), ("sparse", svol.to(dev))):
        for unique in (True, False):
            verts, faces = ref.marching_cubes(vv, 0.0, True, unique)
            torch.cuda.synchronize()
            mc[f"{kind}_{int(unique)}_verts"] = np.array(digest(verts.cpu().numpy()))
            mc[f"{kind}_{int(unique)}_faces"] = np.array(digest(faces.cpu().numpy()))
    np.savez_compressed(out_dir / "ref_mc_sphere.npz", size=np.array([SPHERE_SIZE]), **mc)
    print("fixtures written to", out_dir)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else HERE)
